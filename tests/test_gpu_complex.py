"""Complex shifted-Helmholtz AAR (PETSC_COMPLEX/AAR_Complex.c): complex128 and
complex64 operator and solver against the CPU restatement and the exact FFT
solve; the mixed solver (complex64 iteration, complex128 residual
replacement)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _t(x, dtype=None):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to(device="cuda", dtype=dtype or torch.complex128)


def _cplx_rhs(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.5, 0.5, shape) + 1j * rng.uniform(-0.5, 0.5, shape)


@pytest.mark.parametrize("shape,sigma", [((16, 16, 16), 20 + 15j), ((11, 9, 13), 3.5 + 40j),
                                         ((32, 24, 8), 0.5 + 1j)])
def test_apply_complex(lsg, oracle, shape, sigma):
    import torch
    nz, ny, nx = shape
    x = _cplx_rhs(shape, 1)
    a = -float(nx * nx)
    ref = oracle.apply_c(x, a=a, sigma=sigma)
    op = lsg.Operator((nx, ny, nz), a=a, sigma=sigma)
    scale = (abs(a) * 21.0 + abs(sigma)) * np.abs(x).max()
    y = lsg.apply(op, _t(x)).cpu().numpy()
    assert np.abs(y - ref).max() <= 1e-13 * scale
    y32 = lsg.apply(op, _t(x, torch.complex64)).cpu().numpy()
    assert np.abs(y32 - ref).max() <= 4e-6 * scale


@pytest.mark.parametrize("n,sigma", [(16, 20 + 15j), (24, 2 + 45j), (12, 49 + 1j)])
def test_aar_complex128_matches_restatement(lsg, oracle, n, sigma):
    b = _cplx_rhs((n, n, n), n)
    a = -float(n * n)
    xo, ro = oracle.solve_c(b, a=a, sigma=sigma)
    x, r = lsg.aar(lsg.Operator(n, a=a, sigma=sigma), _t(b))
    assert r["status"] == 0
    assert r["iters"] == ro["iters"]
    assert r["relres"] == pytest.approx(ro["relres"], rel=2e-3)
    x = x.cpu().numpy()
    assert np.linalg.norm(x - xo) <= 1e-8 * np.linalg.norm(xo)
    xf = oracle.fft_solve(b, a=a, sigma=sigma)
    assert np.linalg.norm(x - xf) <= 1e-5 * np.linalg.norm(xf)


def test_complex_with_real_data_equals_real_aar(lsg):
    """Real sigma and real b: the complex AAR takes the real AAR's iterations."""
    import workloads
    n = 20
    b = workloads.uniform_rhs(n, 9)
    op = lsg.Operator(n, a=-400.0, sigma=3.0)
    import torch
    xr, rr = lsg.aar(op, torch.from_numpy(b).cuda())
    xc, rc = lsg.aar(op, _t(b.astype(complex)))
    assert rc["iters"] == rr["iters"]
    assert (xc.real - xr).abs().max().item() <= 1e-9 * xr.abs().max().item()
    assert xc.imag.abs().max().item() == 0.0


@pytest.mark.parametrize("n,sigma", [(32, 20 + 15j), (48, 1.0 + 1.0j)])
def test_aar_mixed_complex(lsg, oracle, n, sigma):
    import torch
    b = _cplx_rhs((n, n, n), 3 * n)
    a = -float(n * n)
    op = lsg.Operator(n, a=a, sigma=sigma)
    x, r = lsg.aar_mixed(op, _t(b), tol=1e-8)
    assert r["status"] == 0 and r["relres"] <= 1e-8
    bt = _t(b)
    true = ((bt - lsg.apply(op, x)).norm() / bt.norm()).item()
    assert true <= 1e-8 * 1.01
    xf = oracle.fft_solve(b, a=a, sigma=sigma)
    lam = np.abs(oracle.symbol((n, n, n), a=a) + sigma)
    kappa = lam.max() / lam.min()  # ||x - x*|| / ||x*|| <= kappa * relres
    assert np.linalg.norm(x.cpu().numpy() - xf) <= kappa * 1e-8 * np.linalg.norm(xf)
    x32, r32 = lsg.aar(op, _t(b, torch.complex64), tol=1e-5)
    assert r32["status"] == 0


def test_petsc_complex_driver_problem(lsg, oracle):
    """PETSC_COMPLEX's own problem: 36^3 (system.c:26-28), A = -(1/(4 pi)) Lap_h
    + Q with Q = -0.134992 - 0.070225i (system.c:217-220, 244), x0 = 1
    (system.c:165), Jacobi (pc = 0), the README's run: tol 1e-6, m = 13, p = 11,
    omega = 1.0, beta = 0.9, max_iter 2000 (main.c:51-52).  PETSc's random
    generator is absent: b has real and imaginary parts U[0, 1) (VecSetRandom's
    range) from seed 36.  The GPU complex AAR must take the restatement's
    iteration count (99) and agree with it and with the FFT solve."""
    import torch
    n = 36
    Q = complex(-0.134992, -0.070225)
    rng = np.random.default_rng(36)
    b = rng.uniform(0, 1, (n, n, n)) + 1j * rng.uniform(0, 1, (n, n, n))
    x0 = np.ones((n, n, n), dtype=np.complex128)
    kw = dict(omega=1.0, beta=0.9, m=13, p=11, tol=1e-6, max_iter=2000)
    xo, ro = oracle.solve_c(b, x0, sigma=Q, **kw)
    op = lsg.Operator(n, sigma=Q)
    x, r = lsg.aar(op, torch.from_numpy(b).cuda(), torch.from_numpy(x0).cuda(), **kw)
    assert ro["converged"] and r["status"] == 0
    assert r["iters"] == ro["iters"], (r, ro)
    assert r["relres"] == pytest.approx(ro["relres"], rel=2e-2)
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - xo) <= 1e-8 * np.linalg.norm(xo)
    xf = oracle.fft_solve(b, sigma=Q)
    lam = np.abs(oracle.symbol((n, n, n), sigma=Q))
    assert np.linalg.norm(xg - xf) <= (lam.max() / lam.min()) * 1e-6 * np.linalg.norm(xf)
    # complex64 inner iteration with complex128 refinement reaches the same tolerance
    xm, rm = lsg.aar_mixed(op, torch.from_numpy(b).cuda(), torch.from_numpy(x0).cuda(), **kw)
    assert rm["status"] == 0 and rm["relres"] <= 1e-6
