"""Full-size (256^3) properties: the solvers reach the requested FP64 residual
(recomputed independently with the device operator) and agree with the FFT
diagonal solve of the periodic operator."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problem256(lsg, oracle):
    import torch
    import workloads
    b = workloads.uniform_rhs(256, 1)
    xf = oracle.fft_solve(b)
    return torch.from_numpy(b).cuda(), xf


def _check(lsg, b, xf, x, r, tol):
    import torch
    op = lsg.Operator(256)
    true = (b - lsg.apply(op, x)).norm().item() / b.norm().item()
    assert r["status"] == 0, r
    assert true <= tol * 1.01, (true, r)
    xm = x - x.mean()
    xft = torch.from_numpy(xf).cuda()
    err = (xm - xft).norm().item() / xft.norm().item()
    return true, err


def _pinned(name):
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "large_256.json")) as f:
        return json.load(f)[name]


def test_aar_fp64_256(lsg, problem256, golden):
    """Same iteration count as the CPU oracle's full run (tests/golden/large_256.json).

    The FP64 stencil passes run in double-float arithmetic (rounding ~2^-48 of
    sum |w| |x| instead of FP64's ~2^-53), which moves the final residual of
    this 1320-iteration trajectory by ~1% (9.52e-9 against the oracle's
    9.43e-9); with FP64 arithmetic (lsg_set_fp64_arith(1)) it stays within
    0.2%."""
    b, xf = problem256
    pinned = _pinned("aar")
    x, r = lsg.aar(lsg.Operator(256), b)
    true, err = _check(lsg, b, xf, x, r, 1e-8)
    assert err < 1e-5
    assert r["iters"] == pinned["iters"]
    assert r["relres"] == pytest.approx(pinned["relres"], rel=2e-2)
    prev = lsg.set_fp64_arith(1)
    try:
        x, r = lsg.aar(lsg.Operator(256), b)
    finally:
        lsg.set_fp64_arith(prev)
    _check(lsg, b, xf, x, r, 1e-8)
    assert r["iters"] == pinned["iters"]
    assert r["relres"] == pytest.approx(pinned["relres"], rel=5e-3)


@pytest.mark.parametrize("solver", ["cg", "pgr", "pl2r"])
def test_fp64_solvers_256(lsg, problem256, solver):
    """The other FP64 solvers at 256^3 to 1e-8 against the oracle's full runs
    (MPI_REAL/CG.c:57-153, PGR.c:90-142, PL2R.c:90-142 restated).

    CG's count is stable under rounding and must match.  PGR and PL2R take
    2500-3600 iterations whose projections amplify last-bit differences: the
    oracle's own count moves with its OpenMP reduction order, and the GPU's
    FP64-arithmetic and double-float runs land within a few periods of it
    (PL2R: 2496 / 2520 against the oracle's 2508), so their counts are held
    to 2%.  Every run must reach the FP64 residual and agree with the FFT
    solve as well as the oracle's solution does (within 2x)."""
    b, xf = problem256
    pinned = _pinned(solver)
    x, r = getattr(lsg, solver)(lsg.Operator(256), b)
    true, err = _check(lsg, b, xf, x, r, 1e-8)
    if solver == "cg":
        assert r["iters"] == pinned["iters"]
    else:
        assert abs(r["iters"] - pinned["iters"]) <= 0.02 * pinned["iters"], (r["iters"], pinned)
    assert err <= 2.0 * pinned["err_vs_fft"] + 1e-9, (err, pinned)


def test_aar_mixed_256(lsg, problem256):
    b, xf = problem256
    x, r = lsg.aar_mixed(lsg.Operator(256), b, tol=1e-8)
    true, err = _check(lsg, b, xf, x, r, 1e-8)
    assert err < 1e-5


def test_mixed_384_blobs(lsg, oracle):
    """384^3 (56.6M unknowns) mixed AAR to 1e-10 on the 64-blob right-hand side
    (width 0.02, seed 3): the FP64 residual recomputed with the device operator
    meets 1e-10 and the solution agrees with the FFT diagonal solve (mean
    removed) within cond * tol."""
    import time
    import torch
    import workloads
    n = 384
    b = workloads.blob_rhs(n, 3)
    op = lsg.Operator(n)
    bt = torch.from_numpy(b).cuda()
    lsg.aar_mixed(op, bt, tol=1e-10)  # warm-up: work arrays, first-launch costs
    torch.cuda.synchronize()
    t0 = time.time()
    x, r = lsg.aar_mixed(op, bt, tol=1e-10)
    torch.cuda.synchronize()
    secs = time.time() - t0
    assert r["status"] == 0 and r["relres"] <= 1e-10
    true = ((bt - lsg.apply(op, x)).norm() / bt.norm()).item()
    assert true <= 1e-10 * 1.01
    lam = torch.from_numpy(oracle.symbol((n, n, n))).cuda()
    bh = torch.fft.fftn(bt)
    lam[0, 0, 0] = 1.0
    xh = bh / lam
    xh[0, 0, 0] = 0.0
    xf = torch.fft.ifftn(xh).real
    err = ((x - x.mean()) - xf).norm().item() / xf.norm().item()
    kappa = (lam.abs().max() / lam.abs()[lam.abs() > 0].min()).item()
    assert err <= kappa * 1e-10
    print(f"384^3 blobs mixed to 1e-10: {secs:.3f} s, {r['iters']} FP32 iterations, "
          f"{r['outer_iters']} FP64 replacements, error vs FFT {err:.2e}")
