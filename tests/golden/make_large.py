"""Pins the iteration counts of the full-size FP64 workload (256^3, U[-0.5,0.5]
seed 1 mean-free, x0 = 0, omega = beta = 0.6, m = 7, p = 6, tol = 1e-8) for
AAR, PGR, PL2R and CG.

    python tests/golden/make_large.py [--threads T] [solver ...]

Runs the CPU oracle (the C restatement of MPI_REAL/{AAR,PGR,PL2R,CG}.c,
OpenMP) once per solver and merges the results into large_256.json (solvers
not named keep their pinned entries).  Besides the iteration count and the
final residual it records the solution's relative error against the FFT
diagonal solve of the periodic operator (mean removed).  bench.py uses the
counts to extrapolate its bounded CPU samples; tests/test_gpu_large.py checks
the GPU solvers against them.  A full run takes several minutes per solver on
8 cores (PGR, the slowest, about 25).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "linear-solver_gb300"))

from oracle import oracle as O  # noqa: E402
import workloads  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "large_256.json")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("solvers", nargs="*", default=["aar", "pgr", "pl2r", "cg"])
    a = ap.parse_args()
    threads = a.threads or O.lib().lsgo_max_threads()
    b = workloads.uniform_rhs(256, 1)
    xf = O.fft_solve(b)
    out = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            out = json.load(f)
    out["workload"] = "256^3 uniform seed 1, x0 = 0, omega=beta=0.6, m=7, p=6, tol=1e-8"
    for s in a.solvers:
        t = time.time()
        x, r = O.solve(s, b, None, threads=threads, omega=0.6, beta=0.6, m=7, p=6, tol=1e-8)
        xm = x - x.mean()
        err = float(np.linalg.norm(xm - xf) / np.linalg.norm(xf))
        out[s] = {"iters": r["iters"], "relres": r["relres"], "err_vs_fft": err,
                  "wall_s": time.time() - t, "threads": threads}
        print(s, out[s], flush=True)
        with open(OUT, "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
