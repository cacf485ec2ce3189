"""The CPU oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the unmodified MPI_REAL sources).

The oracle restates MPI_REAL's arithmetic in the same evaluation order, so the
stencil and coefficients must match bit for bit; the solvers must reproduce the
reference's iteration counts and printed residuals; the pseudo-inverse (a
different SVD algorithm) must agree to rounding.
"""
import numpy as np
import pytest

SOLVERS = ("aar", "pgr", "pl2r", "cg")


def test_coefficients_match_reference_values(oracle):
    c = oracle.coefficients(6)
    # MPI_REAL/system.c:480-498 for FDn = 6
    ref = [-2.982777777777778, 1.7142857142857142, -0.26785714285714285, 0.05291005291005291,
           -0.008928571428571428, 0.001038961038961039, -6.012506012506013e-05]
    assert np.allclose(c, ref, rtol=1e-15, atol=0)


@pytest.mark.parametrize("shape", ["11x17x13", "3x4x5", "1x2x7", "16x16x16"])
def test_stencil_bitwise(oracle, golden, shape):
    g = golden("stencil.npz")
    x = g[f"x_{shape}"]
    assert np.array_equal(oracle.apply(x), g[f"y_{shape}"])
    assert np.array_equal(oracle.apply(x, radius=4, a=1.0), g[f"y4_{shape}"])


def test_pinv_matches_reference(oracle, golden):
    g = golden("pinv.npz")
    for i in range(5):
        A, b, xr = g[f"A{i}"], g[f"b{i}"], g[f"x{i}"]
        x, st = oracle.pinv_solve(A, b)
        assert st == 0
        # two backward-stable SVDs agree to ~cond(A) * eps in the solution
        tol = max(1e-10, 10 * np.linalg.cond(A) * 2.2e-16)
        assert np.linalg.norm(x - xr) <= tol * np.linalg.norm(xr), i


def test_pinv_reference_semantics(oracle):
    """Non-symmetric input: the reference returns V diag(1/w) V^T b, not pinv(A) b."""
    rng = np.random.default_rng(1)
    A = rng.standard_normal((6, 6))
    b = rng.standard_normal(6)
    x, _ = oracle.pinv_solve(A, b)
    _, w, vt = np.linalg.svd(A)
    expect = vt.T @ np.diag(1 / w) @ vt @ b
    assert np.allclose(x, expect, rtol=1e-10)
    assert not np.allclose(x, np.linalg.pinv(A) @ b, rtol=1e-3)


def _check_case(oracle, g, prefix, solver, b, x0=None, **kw):
    x, r = oracle.solve(solver, b, x0, **kw)
    assert r["iters"] == int(g[f"{prefix}_{solver}_iters"]), (prefix, solver)
    # The reference prints relres with %g (6 digits).  The m x m solves use a
    # different SVD algorithm, and with an ill-conditioned history Gram those
    # rounding differences move the final residual by up to ~1e-3 relative.
    assert r["relres"] == pytest.approx(float(g[f"{prefix}_{solver}_relres_printed"]), rel=2e-3)
    key = f"{prefix}_{solver}_x"
    if key in g.files:
        xr = g[key]
        err = np.linalg.norm((x - x.mean()) - (xr - xr.mean())) / np.linalg.norm(xr - xr.mean())
        assert err < 1e-9, (prefix, solver, err)
    return x, r


@pytest.mark.parametrize("solver", SOLVERS)
def test_small_solves(oracle, golden, solver):
    g = golden("small_solves.npz")
    _check_case(oracle, g, "n16", solver, g["b16"])
    _check_case(oracle, g, "odd", solver, g["b_odd"])
    _check_case(oracle, g, "n16_maxit", solver, g["b16"], max_iter=10)
    if solver in ("aar", "cg"):
        _check_case(oracle, g, "tiny", solver, g["b_tiny"])


def test_small_solve_variants(oracle, golden):
    g = golden("small_solves.npz")
    _check_case(oracle, g, "n16_nopc", "pgr", g["b16"], precond=False)
    _check_case(oracle, g, "n16_nopc", "cg", g["b16"], precond=False)
    _check_case(oracle, g, "n16_p1", "aar", g["b16"], p=1, m=3)
    for s in ("aar", "pgr", "pl2r"):
        _check_case(oracle, g, "n16_m3p4", s, g["b16"], m=3, p=4, omega=0.9, beta=0.4)


def test_reference_rhs(oracle, golden):
    g = golden("known_answers_48.npz")
    b = oracle.reference_rhs(48)
    assert np.array_equal(b.reshape(-1)[::97], g["rhs_sample"])


@pytest.mark.parametrize("solver", SOLVERS)
def test_known_answers_48(oracle, golden, solver):
    """MPI_REAL's own driver problem: 48^3, srand RHS, x0 = 1 -> 264 / 390 / 360 / 184."""
    g = golden("known_answers_48.npz")
    b = oracle.reference_rhs(48)
    x, r = oracle.solve(solver, b, np.ones_like(b))
    assert r["iters"] == int(g[f"ref48_{solver}_iters"])
    assert r["iters"] == {"aar": 264, "pgr": 390, "pl2r": 360, "cg": 184}[solver]
    xm = x - x.mean()
    assert np.linalg.norm(xm) == pytest.approx(float(g[f"ref48_{solver}_x_norm"]), rel=1e-9)


def test_fft_oracle_agrees_with_iterative_oracle(oracle):
    import workloads
    b = workloads.uniform_rhs(16, 3)
    x, r = oracle.solve("aar", b, tol=1e-12)
    xf = oracle.fft_solve(b)
    err = np.linalg.norm((x - x.mean()) - xf) / np.linalg.norm(xf)
    assert err < 1e-9
    # shifted operator: the FFT solve is exact for the periodic circulant
    bs = workloads.uniform_rhs(12, 4)
    xs = oracle.fft_solve(bs, a=1.0, sigma=2.5)
    assert np.linalg.norm(oracle.apply(xs, a=1.0, sigma=2.5) - bs) < 1e-12 * np.linalg.norm(bs)


def test_complex_restatement(oracle):
    """Complex AAR: reduces to the pinned real AAR for real data; matches the FFT solve."""
    import workloads
    b = workloads.uniform_rhs(16, 3)
    xr, rr = oracle.solve("aar", b, a=-256.0, sigma=2.0)
    xc, rc = oracle.solve_c(b.astype(complex), a=-256.0, sigma=2.0)
    assert rc["iters"] == rr["iters"]
    assert np.abs(xc - xr).max() < 1e-12
    rng = np.random.default_rng(0)
    bc = rng.uniform(-.5, .5, (12, 12, 12)) + 1j * rng.uniform(-.5, .5, (12, 12, 12))
    xc, rc = oracle.solve_c(bc, a=-144.0, sigma=20 + 15j, tol=1e-12)
    xf = oracle.fft_solve(bc, a=-144.0, sigma=20 + 15j)
    assert np.linalg.norm(xc - xf) <= 1e-10 * np.linalg.norm(xf)
    assert np.linalg.norm(oracle.apply_c(xf, a=-144.0, sigma=20 + 15j) - bc) <= 1e-13 * np.linalg.norm(bc)
