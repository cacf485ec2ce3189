"""The algebra behind the FP32 solver's restructurings, checked in FP64 numpy
on the CPU against the reference-form AAR restatement (oracle.aar_general,
MPI_REAL/AAR.c:37-177):

* the lean form: the Richardson steps carry only the residual recurrence
  r' = r - omega A f and write H = omega f + beta DF, DF; x is rebuilt at each
  extrapolation as x_start + (sum_cycle H_j - beta cf (r - r_start)) + s
  (the cycle's DF columns telescope), and a stop between extrapolations
  folds the cycle's steps in the same way;
* the periodic shifted operator maps the constant vector to sigma times
  itself (the FD Laplacian's rows sum to zero), the identity the mixed
  solver's constant-mode deflation rests on.
"""
import numpy as np
import pytest


def _lean_aar(matvec, cf, b, x0, *, omega, beta, m, p, iters, pinv):
    """AAR in the GPU's lean form (same iteration numbering and columns)."""
    n = b.size
    xs = x0.copy()                      # the cycle-start iterate
    r = b - matvec(xs)
    rs = r.copy()                       # the cycle-start residual
    H, DF = np.zeros((m, n)), np.zeros((m, n))
    last_anderson = 0
    for it in range(1, iters + 1):
        col = (it - 1) % m              # written one launch early (the reference: (it-2) % m at it+1)
        f = cf * r
        if it % p == 0 and it > 1:
            s, _ = pinv(DF @ DF.T, DF @ f)
            step = beta * f - H.T @ s
            mask = [(k - 1) % m for k in range(last_anderson + 1, it)]
            xs = xs + (H[mask].sum(axis=0) - beta * cf * (r - rs)) + step
            rn = r - matvec(step)
            DF[col] = cf * (rn - r)
            H[col] = step + beta * DF[col]
            r = rn
            rs = r.copy()
            last_anderson = it
        else:
            rn = r - omega * matvec(f)
            DF[col] = cf * (rn - r)
            H[col] = omega * f + beta * DF[col]
            r = rn
    mask = [(k - 1) % m for k in range(last_anderson + 1, iters + 1)]
    if mask:                            # stopped between extrapolations: fold the cycle
        xs = xs + (H[mask].sum(axis=0) - beta * cf * (r - rs))
    return xs


@pytest.mark.parametrize("m,p,iters", [(7, 6, 18), (7, 6, 23), (5, 4, 13), (3, 1, 9), (7, 6, 5)])
def test_lean_form_equals_reference_form(oracle, m, p, iters):
    shape = (12, 10, 14)
    rng = np.random.default_rng(7)
    b = rng.uniform(-0.5, 0.5, shape).ravel()
    x0 = rng.uniform(-1, 1, shape).ravel()
    sigma = 1.0
    op = lambda v: oracle.apply(v.reshape(shape), sigma=sigma).ravel()
    diag = oracle.A_REF * 3 * oracle.coefficients(6)[0] + sigma
    cf = 1.0 / diag
    xr, _ = oracle.aar_general(op, np.full(b.size, cf), b, x0, omega=0.6, beta=0.6, m=m, p=p, tol=1e-30,
                               max_iter=iters)
    xl = _lean_aar(op, cf, b, x0, omega=0.6, beta=0.6, m=m, p=p, iters=iters, pinv=oracle.pinv_solve)
    assert np.linalg.norm(xl - xr) <= 1e-11 * np.linalg.norm(xr), (m, p, iters)


@pytest.mark.parametrize("sigma", [0.0, 0.37, 5.0])
def test_periodic_operator_maps_constants_to_sigma(oracle, sigma):
    ones = np.ones((9, 11, 13))
    y = oracle.apply(ones, sigma=sigma)
    assert np.abs(y - sigma).max() <= 1e-13 * max(1.0, abs(oracle.A_REF) * 6 * 3)
