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


def test_aar_fp64_256(lsg, problem256, golden):
    """Same iteration count as the CPU oracle's full run (tests/golden/large_256.json)."""
    import json
    import os
    b, xf = problem256
    x, r = lsg.aar(lsg.Operator(256), b)
    true, err = _check(lsg, b, xf, x, r, 1e-8)
    assert err < 1e-5
    with open(os.path.join(os.path.dirname(__file__), "golden", "large_256.json")) as f:
        pinned = json.load(f)["aar"]
    assert r["iters"] == pinned["iters"]
    assert r["relres"] == pytest.approx(pinned["relres"], rel=5e-3)


def test_aar_mixed_256(lsg, problem256):
    b, xf = problem256
    x, r = lsg.aar_mixed(lsg.Operator(256), b, tol=1e-8)
    true, err = _check(lsg, b, xf, x, r, 1e-8)
    assert err < 1e-5
