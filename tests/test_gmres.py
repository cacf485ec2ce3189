"""Restarted GMRES, the reference's Krylov comparator (PETSc KSPGMRES,
PETSC_REAL/main.c:84-122, restart 30, Jacobi).  The numpy restatement in the
oracle against the FFT solve (CPU), and the GPU GMRES (through the C ABI)
against the restatement: same Arnoldi-step count, same solution to the solve
tolerance times the condition number."""
import numpy as np
import pytest


def test_restatement_solves(oracle):
    n = 12
    rng = np.random.default_rng(4)
    b = rng.uniform(-0.5, 0.5, (n, n, n))
    a = -float(n * n)
    x, r = oracle.gmres(b, restart=30, tol=1e-10, a=a, sigma=2.0, max_iter=5000)
    assert r["converged"]
    xf = oracle.fft_solve(b, a=a, sigma=2.0)
    assert np.linalg.norm(x - xf) <= 1e-7 * np.linalg.norm(xf)
    # restart 5 takes more Arnoldi steps to the same tolerance
    _, r5 = oracle.gmres(b, restart=5, tol=1e-10, a=a, sigma=2.0, max_iter=5000)
    assert r5["converged"] and r5["iters"] > r["iters"]


@pytest.mark.gpu
@pytest.mark.parametrize("n,sigma,restart", [(16, 0.0, 30), (20, 3.0, 10), ((24, 16, 12), 0.5, 30)])
def test_gpu_gmres_matches_restatement(lsg, oracle, n, sigma, restart):
    import torch
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    rng = np.random.default_rng(nx + restart)
    b = rng.uniform(-0.5, 0.5, (nz, ny, nx))
    b -= b.mean()
    a = -float(nx * nx)
    xo, ro = oracle.gmres(b, restart=restart, tol=1e-9, a=a, sigma=sigma, max_iter=4000)
    op = lsg.Operator((nx, ny, nz), a=a, sigma=sigma)
    x, r = lsg.gmres(op, torch.from_numpy(b).cuda(), restart=restart, tol=1e-9, max_iter=4000)
    assert r["status"] == 0 and ro["converged"]
    assert abs(r["iters"] - ro["iters"]) <= 1
    x = x.cpu().numpy()
    if sigma == 0.0:
        x, xo = x - x.mean(), xo - xo.mean()
    assert np.linalg.norm(x - xo) <= 1e-6 * np.linalg.norm(xo)
    x32, r32 = lsg.gmres(op, torch.from_numpy(b).float().cuda(), restart=restart, tol=1e-5, max_iter=4000)
    assert r32["status"] == 0 and r32["relres"] <= 1e-5


@pytest.mark.gpu
def test_gpu_gmres_max_iter(lsg):
    import torch
    n = 16
    b = torch.from_numpy(np.random.default_rng(1).uniform(-0.5, 0.5, (n, n, n))).cuda()
    x, r = lsg.gmres(lsg.Operator(n, a=-256.0, sigma=1.0), b, restart=30, tol=1e-12, max_iter=7)
    assert r["status"] == 1 and r["iters"] == 7
