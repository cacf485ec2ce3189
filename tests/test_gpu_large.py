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


def test_aar_fp64_256(lsg, problem256):
    b, xf = problem256
    x, r = lsg.aar(lsg.Operator(256), b)
    true, err = _check(lsg, b, xf, x, r, 1e-8)
    assert err < 1e-5
    assert r["iters"] % 6 == 0


def test_aar_mixed_256(lsg, problem256):
    b, xf = problem256
    x, r = lsg.aar_mixed(lsg.Operator(256), b, tol=1e-8)
    true, err = _check(lsg, b, xf, x, r, 1e-8)
    assert err < 1e-5
