"""Pins the iteration count of the full-size FP64 AAR workload (256^3, U[-0.5,0.5]
seed 1 mean-free, x0 = 0, omega = beta = 0.6, m = 7, p = 6, tol = 1e-8).

    python tests/golden/make_large.py [threads]

Runs the CPU oracle (the C restatement of MPI_REAL/AAR.c, OpenMP) once and
writes large_256.json.  bench.py uses the count to extrapolate its bounded
CPU sample; tests/test_gpu_large.py checks the GPU solver reaches the same
count.  A full run takes several minutes on 8 cores.
"""
from __future__ import annotations

import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "linear-solver_gb300"))

from oracle import oracle as O  # noqa: E402
import workloads  # noqa: E402


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else O.lib().lsgo_max_threads()
    b = workloads.uniform_rhs(256, 1)
    out = {"workload": "256^3 uniform seed 1, x0 = 0, omega=beta=0.6, m=7, p=6, tol=1e-8",
           "threads": threads}
    for s in ("aar",):
        t = time.time()
        _, r = O.solve(s, b, None, threads=threads, omega=0.6, beta=0.6, m=7, p=6, tol=1e-8)
        out[s] = {"iters": r["iters"], "relres": r["relres"], "wall_s": time.time() - t}
        print(s, out[s], flush=True)
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "large_256.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
