"""The one-warp m x m pseudo-inverse against the reference's PseudoInverseTimesVec."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pinv_matches_reference_golden(lsg, golden):
    import torch
    g = golden("pinv.npz")
    for i in range(5):
        A, b, xr = g[f"A{i}"], g[f"b{i}"], g[f"x{i}"]
        x, st = lsg.pinv_solve(torch.from_numpy(A).cuda(), torch.from_numpy(b).cuda())
        assert st == 0
        tol = max(1e-10, 10 * np.linalg.cond(A) * 2.2e-16)
        assert np.linalg.norm(x.cpu().numpy() - xr) <= tol * np.linalg.norm(xr), i


@pytest.mark.parametrize("m,rank", [(1, 1), (3, 2), (8, 8), (13, 9), (32, 32), (32, 20)])
def test_pinv_sizes(lsg, m, rank):
    import torch
    rng = np.random.default_rng(m + rank)
    F = np.zeros((400, m))
    F[:, :rank] = rng.standard_normal((400, rank))
    A = F.T @ F
    b = rng.standard_normal(m)
    u, w, vt = np.linalg.svd(A)
    keep = w >= m * w.max() * 2.22044605e-16
    expect = vt.T[:, keep] @ np.diag(1 / w[keep]) @ vt[keep] @ b
    x, st = lsg.pinv_solve(torch.from_numpy(A).cuda(), torch.from_numpy(b).cuda())
    assert st == 0
    assert np.allclose(x.cpu().numpy(), expect, rtol=1e-8, atol=1e-10 * np.abs(expect).max())
