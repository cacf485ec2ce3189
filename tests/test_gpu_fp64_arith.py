"""The FP64 solvers' two stencil arithmetics: double-float sums on the FP32 pipe
(the default for tol >= 1e-10) and FP64 arithmetic (lsg_set_fp64_arith(1),
tighter tolerances, lsg_apply).

Both must reproduce the reference's known answers at 48^3 (MPI_REAL driver
problem: 264 / 390 / 360 / 184 iterations).  The double-float residual agrees
with the FP64 operator to ~2^-48 of sum |w| |x|; a value beyond the float
range is reported as LSG_RANGE, and FP64 arithmetic then serves the solve.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KNOWN = {"aar": 264, "pgr": 390, "pl2r": 360, "cg": 184}


@pytest.fixture
def fp64_mode(lsg):
    prev = lsg.set_fp64_arith(0)
    yield lambda m: lsg.set_fp64_arith(m)
    lsg.set_fp64_arith(prev)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("solver", list(KNOWN))
def test_known_answers_both_arithmetics(lsg, oracle, golden, fp64_mode, mode, solver):
    import torch
    fp64_mode(mode)
    g = golden("known_answers_48.npz")
    b = oracle.reference_rhs(48)
    bt = torch.from_numpy(b).cuda()
    x, r = lsg.SOLVERS[solver](lsg.Operator(48), bt, torch.ones_like(bt))
    assert r["status"] == 0 and r["iters"] == KNOWN[solver], (mode, solver, r)
    printed = float(g[f"ref48_{solver}_relres_printed"])
    rtol = 2e-3 if mode == 1 else 2e-2
    assert r["relres"] == pytest.approx(printed, rel=rtol if solver != "cg" else 0.5)
    xm = x.cpu().numpy()
    xm = xm - xm.mean()
    assert np.linalg.norm(xm) == pytest.approx(float(g[f"ref48_{solver}_x_norm"]), rel=1e-8)


def test_small_goldens_fp64_arithmetic(lsg, golden, fp64_mode):
    """The reference's small cases with FP64 arithmetic: printed residuals to 2e-3."""
    from test_gpu_solvers import _case
    fp64_mode(1)
    g = golden("small_solves.npz")
    for solver in KNOWN:
        _case(lsg, g, "n16", solver, g["b16"], rtol=2e-3)
        _case(lsg, g, "odd", solver, g["b_odd"], rtol=2e-3)
    _case(lsg, g, "n16_nopc", "pgr", g["b16"], precond=False, rtol=2e-3)
    _case(lsg, g, "n16_nopc", "cg", g["b16"], precond=False, rtol=2e-3)
    for s in ("aar", "pgr", "pl2r"):
        _case(lsg, g, "n16_m3p4", s, g["b16"], m=3, p=4, omega=0.9, beta=0.4, rtol=2e-3)


@pytest.mark.parametrize("n", [16, 37])
def test_double_float_residual_matches_fp64_operator(lsg, fp64_mode, n):
    """CG with max_iter = 0 returns ||b - A x0|| / ||b|| from its initial
    residual pass (double-float by default; CG.c:65-89 takes the norm before
    the loop); FP64's operator (lsg_apply) gives the reference value.  Random
    x0 of unit size and a small b, so the residual is ~|A x0|."""
    import torch
    g = torch.Generator().manual_seed(5)
    x0 = (torch.rand((n, n, n), generator=g, dtype=torch.float64) - 0.5).cuda()
    b = 1e-3 * (torch.rand((n, n, n), generator=g, dtype=torch.float64) - 0.5).cuda()
    op = lsg.Operator(n)
    ref = ((b - lsg.apply(op, x0)).norm() / b.norm()).item()
    for mode in (0, 1):
        fp64_mode(mode)
        _, r = lsg.cg(op, b, x0.clone(), max_iter=0)
        assert r["relres"] == pytest.approx(ref, rel=1e-12), (mode, r["relres"], ref)


def test_range_beyond_float_reported(lsg, fp64_mode):
    """An initial guess 1e45 times the right-hand side's size cannot be split
    into floats at the solve's scale: the solve stops with LSG_RANGE (raised by
    the binding), and the FP64 arithmetic runs it."""
    import torch
    n = 16
    b = torch.rand((n, n, n), dtype=torch.float64, device="cuda") - 0.5
    b -= b.mean()
    x0 = torch.full_like(b, 1e45)
    x0[0, 0, 0] = -1e45
    with pytest.raises(lsg.CudaLibraryError, match="double-float"):
        lsg.aar(lsg.Operator(n), b, x0.clone(), max_iter=12)
    fp64_mode(1)
    x, r = lsg.aar(lsg.Operator(n), b, x0.clone(), max_iter=12)
    assert r["status"] in (0, 1) and torch.isfinite(x).all()


def test_tight_tolerance_uses_fp64_arithmetic(lsg, fp64_mode):
    """tol below 1e-10 takes FP64 arithmetic even in the default mode: a
    1e-13 solve converges (the double-float floor on this problem is ~1e-13)."""
    import torch
    import workloads
    fp64_mode(0)
    n = 32
    b = torch.from_numpy(workloads.uniform_rhs(n, 4)).cuda()
    op = lsg.Operator(n, a=-float(n * n), sigma=2.0)
    x, r = lsg.aar(op, b, tol=1e-13)
    assert r["status"] == 0 and r["relres"] <= 1e-13
    true = ((b - lsg.apply(op, x)).norm() / b.norm()).item()
    assert true <= 1.5e-13


@pytest.mark.parametrize("n, radius", [(16, 6), (37, 6), (20, 4)])
def test_double_float_complex_residual_matches_fp64_operator(lsg, fp64_mode, n, radius):
    """The complex128 residual replacement of a mixed complex solve in both
    arithmetics: a mixed solve with max_iter = 0 and a nonzero x0 reports
    ||b - A x0|| / ||b|| from its first replacement pass (double-float march by
    default, the shift's imaginary part in the centre weight; radius 4 takes
    the generic-radius march); the complex128 FP64 operator (lsg_apply) gives
    the reference value."""
    import torch
    g = torch.Generator().manual_seed(7)

    def crand(scale):
        re = torch.rand((n, n, n), generator=g, dtype=torch.float64) - 0.5
        im = torch.rand((n, n, n), generator=g, dtype=torch.float64) - 0.5
        return (scale * torch.complex(re, im)).cuda()

    x0 = crand(1.0)
    b = crand(1e-3)
    op = lsg.Operator(n, radius=radius, a=-float(n * n), sigma=complex(3.0, 7.5))
    for mode in (0, 1):
        fp64_mode(mode)
        # with a shift the solve first moves x0's constant mode to mean(b) / sigma
        # and then forms the residual: the returned x is that x0
        x, r = lsg.aar_mixed(op, b, x0.clone(), max_iter=0)
        ref = ((b - lsg.apply(op, x)).norm() / b.norm()).item()
        assert r["relres"] == pytest.approx(ref, rel=1e-12), (mode, r["relres"], ref)


def test_complex_mixed_solve_both_arithmetics(lsg, fp64_mode):
    """A complex mixed solve reaches the same true (complex128) residual with
    the double-float and the FP64-arithmetic residual replacements."""
    import torch
    n = 24
    g = torch.Generator().manual_seed(11)
    b = torch.complex(torch.rand((n, n, n), generator=g, dtype=torch.float64) - 0.5,
                      torch.rand((n, n, n), generator=g, dtype=torch.float64) - 0.5).cuda()
    op = lsg.Operator(n, a=-float(n * n), sigma=complex(2.0, 4.0))
    iters = []
    for mode in (0, 1):
        fp64_mode(mode)
        x, r = lsg.aar_mixed(op, b, tol=1e-9)
        assert r["status"] == 0 and r["relres"] <= 1e-9, (mode, r)
        true = ((b - lsg.apply(op, x)).norm() / b.norm()).item()
        assert true <= 1e-9 * 1.01, (mode, true)
        iters.append(r["iters"])
    assert abs(iters[0] - iters[1]) <= 12, iters
