"""The reference's complex Krylov comparators (PETSC_COMPLEX/main.c:80-175:
KSPGMRES, KSPLGMRES and KSPBICG on the complex-shifted Helmholtz operator;
PETSc is absent, so the oracle restates Saad & Schultz's GMRES with Hermitian
inner products and complex Givens rotations, Baker, Jessup & Manteuffel's
LGMRES, and BiCG in its conjugate orthogonal CG form for the
complex-symmetric operator).  CPU: the restatements against
the FFT solve.  GPU (through the C ABI): against the restatements -- Arnoldi /
COCG step counts within 1, solutions to 1e-6 -- and complex64 runs."""
import numpy as np
import pytest


def _problem(n, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.5, 0.5, (n, n, n)) + 1j * rng.uniform(-0.5, 0.5, (n, n, n))


@pytest.mark.parametrize("sigma", [20 + 10j, 3 + 40j])
def test_restatements_solve(oracle, sigma):
    n = 12
    b = _problem(n, 3)
    a = -float(n * n)
    xf = oracle.fft_solve(b, a=a, sigma=sigma)
    for fn, kw in ((oracle.gmres_c, dict(restart=30, max_iter=5000)), (oracle.cocg, {})):
        x, r = fn(b, a=a, sigma=sigma, tol=1e-10, **kw)
        assert r["converged"], (fn.__name__, r)
        assert np.linalg.norm(x - xf) <= 1e-7 * np.linalg.norm(xf), fn.__name__


def test_complex_gmres_on_real_data_is_real_gmres(oracle):
    n = 10
    b = np.random.default_rng(5).uniform(-0.5, 0.5, (n, n, n))
    b -= b.mean()
    x1, r1 = oracle.gmres(b, tol=1e-8)
    x2, r2 = oracle.gmres_c(b + 0j, tol=1e-8)
    assert r1["iters"] == r2["iters"]
    assert np.abs(x1 - x2.real).max() <= 1e-12 * np.abs(x1).max()


def test_lgmres_restatement(oracle):
    """LGMRES with no augmentation is GMRES (same steps, same iterate); with
    PETSc's default augmentation it solves the real and complex problems."""
    n = 12
    rng = np.random.default_rng(11)
    b = rng.uniform(-0.5, 0.5, (n, n, n))
    b -= b.mean()
    a = -float(n * n)
    x1, r1 = oracle.gmres(b, restart=20, tol=1e-9, a=a, sigma=2.0)
    x0, r0 = oracle.lgmres(b, restart=20, aug=0, tol=1e-9, a=a, sigma=2.0)
    assert r0["iters"] == r1["iters"] and np.array_equal(x0, x1)
    for bb, sg in ((b, 2.0), (_problem(n, 4), 20 + 10j), (_problem(n, 5), 3 + 40j)):
        x, r = oracle.lgmres(bb, restart=30, aug=2, tol=1e-10, a=a, sigma=sg, max_iter=5000)
        xf = oracle.fft_solve(bb, a=a, sigma=sg)
        assert r["converged"] and np.linalg.norm(x - xf) <= 1e-7 * np.linalg.norm(xf)


@pytest.mark.gpu
@pytest.mark.parametrize("n,sigma,restart,aug", [(16, 20 + 10j, 30, 2), (20, 3 + 40j, 12, 3), ((24, 16, 12), 2.0, 30, 2),
                                                 (16, 0.5, 10, 1)])
def test_gpu_lgmres_matches_restatement(lsg, oracle, n, sigma, restart, aug):
    """LGMRES(m, k) (the reference's KSPLGMRES, PETSC_COMPLEX/main.c:123-147)
    against the restatement: operator applications within 1, solution to 1e-6,
    real and complex; complex64 / FP32 runs converge."""
    import torch
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    rng = np.random.default_rng(nx + 7 * restart)
    cx = isinstance(sigma, complex)
    b = rng.uniform(-0.5, 0.5, (nz, ny, nx))
    if cx:
        b = b + 1j * rng.uniform(-0.5, 0.5, (nz, ny, nx))
    else:
        b -= b.mean()
    a = -float(nx * nx)
    xo, ro = oracle.lgmres(b, restart=restart, aug=aug, tol=1e-9, a=a, sigma=sigma, max_iter=4000)
    op = lsg.Operator((nx, ny, nz), a=a, sigma=sigma)
    x, r = lsg.lgmres(op, torch.from_numpy(b).cuda(), restart=restart, aug=aug, tol=1e-9, max_iter=4000)
    assert r["status"] == 0 and ro["converged"]
    assert abs(r["iters"] - ro["iters"]) <= 1, (r, ro)
    assert np.linalg.norm(x.cpu().numpy() - xo) <= 1e-6 * np.linalg.norm(xo)
    lo = torch.complex64 if cx else torch.float32
    x32, r32 = lsg.lgmres(op, torch.from_numpy(b).to(lo).cuda(), restart=restart, aug=aug, tol=1e-5, max_iter=4000)
    assert r32["status"] == 0 and r32["relres"] <= 1e-5


@pytest.mark.gpu
def test_gpu_lgmres_rejects_bad_augmentation(lsg):
    import torch
    op = lsg.Operator(8, a=-64.0, sigma=1.0)
    b = torch.ones((8, 8, 8), dtype=torch.float64, device="cuda")
    for aug, restart in ((5, 30), (10, 10), (-1, 30)):
        with pytest.raises(lsg.CudaLibraryError):
            lsg.lgmres(op, b, restart=restart, aug=aug)


@pytest.mark.gpu
@pytest.mark.parametrize("n,sigma,restart", [(16, 20 + 10j, 30), (20, 3 + 40j, 10), ((24, 16, 12), 8 + 2j, 30)])
def test_gpu_complex_gmres_matches_restatement(lsg, oracle, n, sigma, restart):
    import torch
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    rng = np.random.default_rng(nx + restart)
    b = rng.uniform(-0.5, 0.5, (nz, ny, nx)) + 1j * rng.uniform(-0.5, 0.5, (nz, ny, nx))
    a = -float(nx * nx)
    xo, ro = oracle.gmres_c(b, restart=restart, tol=1e-9, a=a, sigma=sigma, max_iter=4000)
    op = lsg.Operator((nx, ny, nz), a=a, sigma=sigma)
    x, r = lsg.gmres(op, torch.from_numpy(b).cuda(), restart=restart, tol=1e-9, max_iter=4000)
    assert r["status"] == 0 and ro["converged"]
    assert abs(r["iters"] - ro["iters"]) <= 1, (r, ro)
    x = x.cpu().numpy()
    assert np.linalg.norm(x - xo) <= 1e-6 * np.linalg.norm(xo)
    x64, r64 = lsg.gmres(op, torch.from_numpy(b).to(torch.complex64).cuda(), restart=restart, tol=1e-5,
                         max_iter=4000)
    assert r64["status"] == 0 and r64["relres"] <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("n,sigma", [(16, 20 + 10j), (20, 3 + 40j), ((24, 16, 12), 8 + 2j)])
def test_gpu_cocg_matches_restatement(lsg, oracle, n, sigma):
    import torch
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    rng = np.random.default_rng(nx + 1)
    b = rng.uniform(-0.5, 0.5, (nz, ny, nx)) + 1j * rng.uniform(-0.5, 0.5, (nz, ny, nx))
    a = -float(nx * nx)
    xo, ro = oracle.cocg(b, tol=1e-9, a=a, sigma=sigma)
    op = lsg.Operator((nx, ny, nz), a=a, sigma=sigma)
    x, r = lsg.cocg(op, torch.from_numpy(b).cuda(), tol=1e-9)
    assert r["status"] == 0 and ro["converged"]
    assert abs(r["iters"] - ro["iters"]) <= 1, (r, ro)
    assert np.linalg.norm(x.cpu().numpy() - xo) <= 1e-6 * np.linalg.norm(xo)
    xf = oracle.fft_solve(b, a=a, sigma=sigma)
    assert np.linalg.norm(x.cpu().numpy() - xf) <= 1e-6 * np.linalg.norm(xf)
    x64, r64 = lsg.cocg(op, torch.from_numpy(b).to(torch.complex64).cuda(), tol=1e-5)
    assert r64["status"] == 0 and r64["relres"] <= 1e-5


@pytest.mark.gpu
def test_gpu_cocg_rejects_real(lsg):
    import torch
    b = torch.zeros((8, 8, 8), dtype=torch.float64, device="cuda")
    with pytest.raises(lsg.CudaLibraryError):
        lsg.cocg(lsg.Operator(8), b)


@pytest.mark.gpu
def test_gpu_gmres_workspaces_per_dtype(lsg):
    """FP64 and complex64 vectors have the same element size but different
    GMRES states: solves of both (and complex128) on one grid and restart
    length, interleaved in one process, each converge."""
    import torch
    n = 12
    rng = np.random.default_rng(4)
    br = rng.uniform(-0.5, 0.5, (n, n, n))
    bc = br + 1j * rng.uniform(-0.5, 0.5, (n, n, n))
    opr = lsg.Operator(n, a=-float(n * n), sigma=2.0)
    opc = lsg.Operator(n, a=-float(n * n), sigma=2.0 + 3.0j)
    for dt, b, op in [(torch.float64, br, opr), (torch.complex64, bc, opc), (torch.complex128, bc, opc),
                      (torch.float64, br, opr), (torch.complex64, bc, opc)]:
        x, r = lsg.gmres(op, torch.from_numpy(b).to(device="cuda", dtype=dt), restart=20,
                         tol=1e-5 if dt == torch.complex64 else 1e-8)
        assert r["status"] == 0, (dt, r)
