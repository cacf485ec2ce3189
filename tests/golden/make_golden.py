"""Writes the golden fixtures in this folder from the UNMODIFIED reference.

Run in a checkout that has the reference sources (default
``/root/reference/MPI_REAL``; override with ``LSG_REFERENCE_DIR``):

    python tests/golden/make_golden.py

It compiles the reference (``make -C oracle ref``: the reference's own C
files against a one-rank MPI shim), runs its solvers / stencil / pseudo-inverse
through ``oracle/ref_harness.c`` and stores inputs and outputs as ``.npz``.
The reference prints its relative residual with ``%g`` (6 significant
digits), so ``relres_printed`` keeps that text value; ``true_relres`` is the
full-precision ``||b - A x|| / ||b||`` of the returned solution, evaluated with
the reference's own operator.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "linear-solver_gb300"))

from oracle import oracle as O  # noqa: E402
import workloads  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
SOLVERS = ("aar", "pgr", "pl2r", "cg")


def ref_apply(x, radius=6, a=O.A_REF):
    nz, ny, nx = x.shape
    y = np.empty(x.size)
    O.ref().refh_apply(nx, ny, nz, radius, a, np.ascontiguousarray(x).reshape(-1).copy(), y)
    return y.reshape(x.shape)


def true_relres(x, b):
    return float(np.linalg.norm(b - ref_apply(x)) / np.linalg.norm(b))


def solve_all(prefix, b, x0, out, solvers=SOLVERS, keep_x=False, **kw):
    for s in solvers:
        x, r = O.ref_solve(s, b, x0, **kw)
        out[f"{prefix}_{s}_iters"] = r["iters"]
        out[f"{prefix}_{s}_relres_printed"] = r["relres"]
        out[f"{prefix}_{s}_true_relres"] = true_relres(x, b)
        xm = x - x.mean()
        out[f"{prefix}_{s}_x_mean"] = x.mean()
        out[f"{prefix}_{s}_x_norm"] = np.linalg.norm(xm)
        out[f"{prefix}_{s}_x_sample"] = xm.reshape(-1)[::97].copy()
        if keep_x:
            out[f"{prefix}_{s}_x"] = x
        print(prefix, s, r["iters"], r["relres"])


def main():
    O.build(with_ref=True)
    if not O.ref_available():
        raise SystemExit("reference build missing")

    # (1) the reference driver's own problem: 48^3, its srand RHS, x0 = 1, `1e-8 7 6 0.6 0.6`.
    out = {}
    b = O.reference_rhs(48)
    br = np.empty(48 ** 3)
    O.ref().refh_rhs(48, 48, 48, 6, br)
    assert np.array_equal(b.reshape(-1), br)
    out["rhs_sample"] = b.reshape(-1)[::97].copy()
    solve_all("ref48", b, np.ones_like(b), out)
    np.savez_compressed(os.path.join(OUT, "known_answers_48.npz"), **out)

    # (2) workload 1: 48^3, U[-0.5,0.5] seed 0 mean-free, x0 = 0.
    out = {}
    b = workloads.uniform_rhs(48, 0)
    out["rhs_sample"] = b.reshape(-1)[::97].copy()
    solve_all("cfg1", b, None, out)
    np.savez_compressed(os.path.join(OUT, "config1_48.npz"), **out)

    # (3) small grids with full solutions.
    out = {}
    b16 = workloads.uniform_rhs(16, 3)
    out["b16"] = b16
    solve_all("n16", b16, None, out, keep_x=True)
    solve_all("n16_nopc", b16, None, out, solvers=("pgr", "cg"), keep_x=True, precond=False)
    solve_all("n16_p1", b16, None, out, solvers=("aar",), keep_x=True, p=1, m=3)
    solve_all("n16_m3p4", b16, None, out, solvers=("aar", "pgr", "pl2r"), keep_x=True, m=3, p=4,
              omega=0.9, beta=0.4)
    b_odd = workloads.uniform_rhs((12, 10, 8), 7)
    out["b_odd"] = b_odd
    solve_all("odd", b_odd, None, out, keep_x=True)
    b_tiny = workloads.uniform_rhs((5, 7, 9), 8)
    out["b_tiny"] = b_tiny
    solve_all("tiny", b_tiny, None, out, solvers=("aar", "cg"), keep_x=True)
    # max_iter exhausted: the reference prints the last residual it computed.
    solve_all("n16_maxit", b16, None, out, solvers=SOLVERS, keep_x=True, max_iter=10)
    np.savez_compressed(os.path.join(OUT, "small_solves.npz"), **out)

    # (4) the stencil on odd and smaller-than-radius grids.
    out = {}
    rng = np.random.default_rng(5)
    for shape in ((11, 17, 13), (3, 4, 5), (1, 2, 7), (16, 16, 16)):
        x = rng.uniform(-1, 1, size=shape)
        key = "x".join(map(str, shape))
        out[f"x_{key}"] = x
        out[f"y_{key}"] = ref_apply(x)
        out[f"y4_{key}"] = ref_apply(x, radius=4, a=1.0)
    np.savez_compressed(os.path.join(OUT, "stencil.npz"), **out)

    # (5) the m x m pseudo-inverse: rank-deficient Gram (first Anderson step), full-rank,
    #     ill-conditioned and non-symmetric (PGR's DX^T DF) cases.
    out = {}
    rng = np.random.default_rng(6)
    cases = []
    F = np.zeros((200, 7))
    F[:, :5] = rng.standard_normal((200, 5))
    cases.append(F.T @ F)
    F = rng.standard_normal((200, 7))
    cases.append(F.T @ F)
    U, _ = np.linalg.qr(rng.standard_normal((7, 7)))
    cases.append(U @ np.diag(np.logspace(0, -13, 7)) @ U.T)
    cases.append(rng.standard_normal((7, 7)))
    X = rng.standard_normal((300, 5))
    cases.append(X.T @ (X + 0.1 * rng.standard_normal((300, 5))))
    for i, A in enumerate(cases):
        bb = rng.standard_normal(A.shape[0])
        out[f"A{i}"] = A
        out[f"b{i}"] = bb
        out[f"x{i}"] = O.ref_pinv(A, bb)
    np.savez_compressed(os.path.join(OUT, "pinv.npz"), **out)
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
