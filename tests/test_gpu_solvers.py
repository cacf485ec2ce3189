"""Solver parity: the GPU solvers against the reference's own runs (golden
fixtures from the unmodified MPI_REAL code) and the CPU oracle.

FP64 bar: identical iteration counts, the reference's printed residual to
2e-2 relative, and the solution (mean removed, since the periodic Poisson
operator is singular) to 1e-8 relative.  The FP64 solvers' stencil sums run
in double-float arithmetic by default (rounding ~2^-48 of sum |w| |x|, 30x
FP64's), which moves the residual at the last check of a long trajectory by
up to ~1.5% (PGR without preconditioning at 16^3); with FP64 arithmetic the
same cases hold 2e-3 (tests/test_gpu_fp64_arith.py).

CG's final residual is compared more loosely (within 50%, and below tol):
the reference's CG restarts the residual every 50 steps but keeps the old
search direction (MPI_REAL/CG.c:109-150), and near convergence that recurrence
amplifies last-bit differences (here: parallel instead of serial sums) by
roughly 10x per iteration, so the printed residual at the stopping iteration
is only reproducible by running the reference's own serial arithmetic (the
CPU oracle does, bit for bit).  Iteration counts and solutions still match.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SOLVERS = ("aar", "pgr", "pl2r", "cg")


def _t(x, dtype=None):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to(device="cuda", dtype=dtype or torch.float64)


def _merr(x, xr):
    x = x - x.mean()
    xr = xr - xr.mean()
    return np.linalg.norm(x - xr) / np.linalg.norm(xr)


def _case(lsg, g, prefix, solver, b, x0=None, rtol=2e-2, **kw):
    op_kw = {k: kw.pop(k) for k in ("precond",) if k in kw}
    nz, ny, nx = b.shape
    op = lsg.Operator((nx, ny, nz), **op_kw)
    x, r = lsg.SOLVERS[solver](op, _t(b), None if x0 is None else _t(x0), **kw)
    x = x.cpu().numpy()
    assert r["iters"] == int(g[f"{prefix}_{solver}_iters"]), (prefix, solver, r)
    printed = float(g[f"{prefix}_{solver}_relres_printed"])
    assert r["relres"] == pytest.approx(printed, rel=rtol if solver != "cg" else 0.5)
    if printed <= kw.get("tol", 1e-8):
        assert r["relres"] <= kw.get("tol", 1e-8)
    key = f"{prefix}_{solver}_x"
    if key in g.files:
        assert _merr(x, g[key]) < 1e-8, (prefix, solver)
    return x, r


@pytest.mark.parametrize("solver", SOLVERS)
def test_small_golden(lsg, golden, solver):
    g = golden("small_solves.npz")
    _case(lsg, g, "n16", solver, g["b16"])
    _case(lsg, g, "odd", solver, g["b_odd"])
    _case(lsg, g, "n16_maxit", solver, g["b16"], max_iter=10)
    if solver in ("aar", "cg"):
        _case(lsg, g, "tiny", solver, g["b_tiny"])


def test_small_golden_variants(lsg, golden):
    g = golden("small_solves.npz")
    _case(lsg, g, "n16_nopc", "pgr", g["b16"], precond=False)
    _case(lsg, g, "n16_nopc", "cg", g["b16"], precond=False)
    _case(lsg, g, "n16_p1", "aar", g["b16"], p=1, m=3)
    for s in ("aar", "pgr", "pl2r"):
        _case(lsg, g, "n16_m3p4", s, g["b16"], m=3, p=4, omega=0.9, beta=0.4)


@pytest.mark.parametrize("solver", SOLVERS)
def test_known_answers_48(lsg, oracle, golden, solver):
    """MPI_REAL's driver problem (48^3, srand RHS, x0 = 1): 264 / 390 / 360 / 184 iterations."""
    g = golden("known_answers_48.npz")
    b = oracle.reference_rhs(48)
    x, r = _case(lsg, g, "ref48", solver, b, np.ones_like(b))
    assert r["iters"] == {"aar": 264, "pgr": 390, "pl2r": 360, "cg": 184}[solver]
    xm = x - x.mean()
    assert np.linalg.norm(xm) == pytest.approx(float(g[f"ref48_{solver}_x_norm"]), rel=1e-8)
    assert np.allclose(xm.reshape(-1)[::97], g[f"ref48_{solver}_x_sample"], rtol=0,
                       atol=1e-8 * np.abs(xm).max())


@pytest.mark.parametrize("solver", SOLVERS)
def test_workload1_48(lsg, golden, solver):
    """48^3, U[-0.5,0.5] seed 0, x0 = 0."""
    import workloads
    g = golden("config1_48.npz")
    b = workloads.uniform_rhs(48, 0)
    _case(lsg, g, "cfg1", solver, b)


@pytest.mark.parametrize("solver", ("aar", "pgr", "pl2r"))
def test_long_history_generic_path(lsg, oracle, solver):
    """m = 13, p = 11 (the reference README's example) exercises the m > 8 Gram path."""
    import workloads
    b = workloads.uniform_rhs(20, 11)
    kw = dict(m=13, p=11, omega=1.0, beta=0.9, tol=1e-8)
    xo, ro = oracle.solve(solver, b, **kw)
    x, r = lsg.SOLVERS[solver](lsg.Operator(20), _t(b), **kw)
    assert r["iters"] == ro["iters"]
    assert _merr(x.cpu().numpy(), xo) < 1e-7


@pytest.mark.parametrize("solver", SOLVERS)
def test_other_radius_and_shift(lsg, oracle, solver):
    """FDn = 4 with a positive diagonal shift (generic stencil path, SPD operator)."""
    import workloads
    b = workloads.uniform_rhs((18, 14, 11), 12)
    xo, ro = oracle.solve(solver, b, radius=4, a=-0.3, sigma=0.05)
    op = lsg.Operator((18, 14, 11), radius=4, a=-0.3, sigma=0.05)
    x, r = lsg.SOLVERS[solver](op, _t(b))
    assert r["iters"] == ro["iters"]
    xr = xo
    assert np.linalg.norm(x.cpu().numpy() - xr) / np.linalg.norm(xr) < 1e-8


def test_compat_entry_points_on_host_buffers(lsg, golden):
    """The reference-prototype AAR/PGR/PL2R/CG(POISSON*, ...) on host arrays."""
    g = golden("small_solves.npz")
    for s in SOLVERS:
        x = np.zeros((16, 16, 16))
        b = np.ascontiguousarray(g["b16"])
        r = lsg.compat_solve(s, x, b)
        assert r["last_status"] == 0
        assert r["iters"] == int(g[f"n16_{s}_iters"])
        assert _merr(x, g[f"n16_{s}_x"]) < 1e-8


def test_fp32_solvers_converge(lsg, oracle):
    import torch
    import workloads
    b = workloads.uniform_rhs(32, 5)
    xf = oracle.fft_solve(b)
    for s in SOLVERS:
        x, r = lsg.SOLVERS[s](lsg.Operator(32), _t(b, torch.float32), tol=1e-5)
        assert r["status"] == 0, (s, r)
        # relres 1e-5 bounds the error by cond(D^-1 A) * 1e-5 (cond ~ 550 at 32^3)
        assert _merr(x.double().cpu().numpy(), xf) < 5e-3, s


@pytest.mark.parametrize("m,p,k", [(7, 6, 17), (7, 6, 18), (7, 6, 5), (3, 6, 17), (3, 1, 9), (5, 4, 13)])
def test_fp32_iterate_at_max_iter(lsg, oracle, m, p, k):
    """The FP32 AAR iterate after k iterations against the oracle's FP64
    iterate: k between extrapolations (the Richardson passes of a lean solve
    leave x out, so the stop folds the cycle's steps into x), k at an
    extrapolation, p - 1 > m (the recurrence keeps x in its passes), p = 1."""
    import torch
    import workloads
    b = workloads.uniform_rhs(24, 3)
    x0 = np.random.default_rng(4).uniform(-1, 1, b.shape)
    xr, _ = oracle.solve("aar", b, x0, m=m, p=p, max_iter=k, tol=1e-30)
    x, r = lsg.aar(lsg.Operator(24), _t(b, torch.float32), _t(x0, torch.float32), m=m, p=p, max_iter=k,
                   tol=1e-30)
    assert r["status"] != 0  # stopped by max_iter
    x = x.double().cpu().numpy()
    assert np.linalg.norm(x - xr) <= 2e-5 * np.linalg.norm(xr), (m, p, k)


@pytest.mark.parametrize("sigma", [0.1, 0.3 + 0.2j])
def test_mixed_deflates_constant_mode(lsg, oracle, sigma):
    """Shifted operator, right-hand side with a non-zero mean: the constant
    mode (eigenvalue sigma, the slowest one when sigma is small) is set
    exactly at every FP64 replacement, so the FP32 iteration never has to
    resolve it.  Without that it plateaus at the mean's share of the residual
    and needs 15-50 replacements; here a few suffice."""
    import torch
    n = 48
    rng = np.random.default_rng(11)
    b = rng.standard_normal((n, n, n)) + 0.05
    if isinstance(sigma, complex):
        b = b + 1j * (rng.standard_normal((n, n, n)) - 0.03)
    op = lsg.Operator(n, a=-float(n * n), sigma=sigma)
    bt = torch.from_numpy(b).cuda()
    x, r = lsg.aar_mixed(op, bt, tol=1e-10)
    assert r["status"] == 0 and r["outer_iters"] <= 6, r
    res = (bt - lsg.apply(op, x)).norm() / bt.norm()
    assert res.item() <= 1e-10 * 1.01
    xf = oracle.fft_solve(b, a=-float(n * n), sigma=sigma)
    lam = np.abs(oracle.symbol(b.shape, a=-float(n * n)) + sigma)
    kappa = lam.max() / lam.min()
    assert np.linalg.norm(x.cpu().numpy() - xf) <= kappa * 1e-10 * np.linalg.norm(xf)
    assert abs(x.mean().item() - b.mean() / sigma) <= 1e-9 * abs(b.mean() / sigma)


@pytest.mark.parametrize("sigma", [0.0, 2.0])
def test_mixed_initial_guess(lsg, oracle, sigma):
    """x0 = 0 starts from r = b without a stencil pass (b - sigma c after the
    constant-mode deflation); a non-zero x0 takes the FP64 residual.  Both
    converge to the same solution."""
    import torch
    import workloads
    n = 40
    b = workloads.uniform_rhs(n, 21)
    b = b - b.mean()
    op = lsg.Operator(n, sigma=sigma)
    bt = _t(b)
    x0 = _t(np.random.default_rng(3).uniform(-1, 1, b.shape))
    xa, ra = lsg.aar_mixed(op, bt, tol=1e-10)
    xb, rb = lsg.aar_mixed(op, bt, x0, tol=1e-10)
    for x, r in ((xa, ra), (xb, rb)):
        assert r["status"] == 0, r
        assert ((bt - lsg.apply(op, x)).norm() / bt.norm()).item() <= 1e-10 * 1.01
    if sigma == 0.0:
        assert _merr(xa.cpu().numpy(), xb.cpu().numpy()) < 1e-6
    else:
        assert ((xa - xb).norm() / xa.norm()).item() < 1e-6


def test_mixed_precision_to_1e10(lsg, oracle):
    import workloads
    b = workloads.uniform_rhs(48, 0)
    x, r = lsg.aar_mixed(lsg.Operator(48), _t(b), tol=1e-10)
    assert r["status"] == 0 and r["relres"] <= 1e-10, r
    assert r["outer_iters"] >= 2
    xf = oracle.fft_solve(b)
    assert _merr(x.cpu().numpy(), xf) < 1e-7
    # the FP64 residual, recomputed independently
    op = lsg.Operator(48)
    xt = x
    res = _t(b) - lsg.apply(op, xt)
    assert res.norm().item() / np.linalg.norm(b) <= 1e-10


def test_nan_rhs_reported_not_faulting(lsg):
    import torch
    b = torch.zeros((16, 16, 16), dtype=torch.float64, device="cuda")
    b[3, 4, 5] = float("nan")
    for s in SOLVERS:
        x, r = lsg.SOLVERS[s](lsg.Operator(16), b)
        assert r["status"] == 2, (s, r)
    x, r = lsg.aar_mixed(lsg.Operator(16), b)
    assert r["status"] == 2


def test_zero_iterations(lsg):
    import torch
    b = torch.ones((8, 8, 8), dtype=torch.float64, device="cuda")
    x, r = lsg.aar(lsg.Operator(8), b - b.mean(), max_iter=0)
    assert r["iters"] == 0 and r["status"] == 1
    x, r = lsg.cg(lsg.Operator(8), b - b.mean(), max_iter=0)
    assert r["iters"] == 0


@pytest.mark.parametrize("dtype_name", ["float64", "float32"])
def test_unaligned_views(lsg, dtype_name):
    """x and b as views at a one-element offset (not 16-byte aligned): the
    16-byte load paths stand aside (the scalar paths compute the same sums),
    so the solve matches the one on aligned copies."""
    import torch
    dt = getattr(torch, dtype_name)
    n = 24
    rng = np.random.default_rng(12)
    b = rng.uniform(-0.5, 0.5, (n, n, n))
    b -= b.mean()
    op = lsg.Operator(n, a=-float(n * n), sigma=1.0)
    tol = 1e-9 if dt == torch.float64 else 1e-5
    bb = torch.from_numpy(b).to(device="cuda", dtype=dt)
    x_ref, r_ref = lsg.aar(op, bb, tol=tol)
    store_b = torch.empty(n ** 3 + 1, dtype=dt, device="cuda")
    store_x = torch.zeros(n ** 3 + 1, dtype=dt, device="cuda")
    bv = store_b[1:].view(n, n, n)
    bv.copy_(bb)
    xv = store_x[1:].view(n, n, n)
    assert bv.data_ptr() % 16 != 0 and xv.data_ptr() % 16 != 0
    import ctypes as C
    res = lsg._Result()
    prm = lsg._params(tol=tol)
    rc = lsg.lib().lsg_aar(C.byref(op._s), C.byref(prm), lsg._dtype_code(bv), C.c_void_p(xv.data_ptr()),
                           C.c_void_p(bv.data_ptr()), C.byref(res), lsg._stream_ptr())
    torch.cuda.synchronize()
    r = lsg._result(res)
    assert rc == 0 and r["iters"] == r_ref["iters"]
    assert ((xv - x_ref).norm() / x_ref.norm()).item() <= (1e-12 if dt == torch.float64 else 1e-6)
