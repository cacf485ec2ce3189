"""The device operator y = (a*Lap + sigma) x against the reference and oracle.

FP64: the kernel sums in a different order (pair sums, FMA), so it agrees
with the reference to a few ulps of sum_p |w_p| |x| (tested at 1e-13
relative).  FP32: against the FP64 result at 2e-6 relative to the same scale.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scale(x, op_coeff, a, sigma=0.0):
    return (abs(a) * (3 * abs(op_coeff[0]) + 6 * sum(abs(c) for c in op_coeff[1:])) + abs(sigma)) * np.abs(x).max()


def _dev(lsg, x, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to(device="cuda", dtype=dtype)


@pytest.mark.parametrize("shape", ["11x17x13", "3x4x5", "1x2x7", "16x16x16"])
def test_apply_matches_reference_golden(lsg, golden, shape):
    import torch
    g = golden("stencil.npz")
    x = g[f"x_{shape}"]
    nz, ny, nx = x.shape
    for radius, a, key in ((6, lsg.A_REF, "y"), (4, 1.0, "y4")):
        op = lsg.Operator((nx, ny, nz), radius=radius, a=a)
        y = lsg.apply(op, _dev(lsg, x, torch.float64)).cpu().numpy()
        s = _scale(x, op.coeff, a)
        assert np.abs(y - g[f"{key}_{shape}"]).max() <= 1e-13 * s
        y32 = lsg.apply(op, _dev(lsg, x, torch.float32)).cpu().numpy()
        assert np.abs(y32 - g[f"{key}_{shape}"]).max() <= 2e-6 * s


@pytest.mark.parametrize("shape,radius,sigma", [((32, 32, 32), 6, 0.0), ((64, 48, 40), 6, 1.5),
                                                ((33, 17, 70), 6, 0.0), ((256, 8, 5), 6, 0.0),
                                                ((20, 21, 22), 1, 0.0), ((20, 21, 22), 2, 3.0),
                                                ((20, 21, 22), 3, 0.0), ((19, 9, 40), 5, 0.0),
                                                ((24, 24, 24), 7, 0.0), ((24, 24, 24), 8, -2.0),
                                                ((7, 5, 3), 8, 0.0)])
def test_apply_matches_oracle(lsg, oracle, shape, radius, sigma):
    import torch
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 7 + radius)
    x = rng.uniform(-1, 1, size=(nz, ny, nx))
    op = lsg.Operator(shape, radius=radius, sigma=sigma)
    ref = oracle.apply(x, radius=radius, a=op.a, sigma=sigma)
    s = _scale(x, op.coeff, op.a, sigma)
    y = lsg.apply(op, _dev(lsg, x, torch.float64)).cpu().numpy()
    assert np.abs(y - ref).max() <= 1e-13 * s
    y32 = lsg.apply(op, _dev(lsg, x, torch.float32)).cpu().numpy()
    assert np.abs(y32 - ref).max() <= 2e-6 * s


def test_apply_256_linearity_and_fft_symbol(lsg, oracle):
    """Full size: A applied to a Fourier mode returns symbol * mode (exact
    eigenvector of the periodic operator), and A is linear."""
    import torch
    n = 256
    op = lsg.Operator(n)
    k = (3, 5, 7)
    ax = [2 * np.pi * k[d] * torch.arange(n, dtype=torch.float64, device="cuda") / n for d in range(3)]
    mode = (torch.cos(ax[2])[:, None, None] * torch.cos(ax[1])[None, :, None]
            * torch.cos(ax[0])[None, None, :]).contiguous()
    lam = oracle.symbol((n, n, n))[k[2], k[1], k[0]]
    y = lsg.apply(op, mode)
    assert torch.max(torch.abs(y - lam * mode)).item() < 1e-13
    g = torch.Generator(device="cuda").manual_seed(0)
    u = torch.rand((n, n, n), dtype=torch.float64, device="cuda", generator=g)
    v = torch.rand((n, n, n), dtype=torch.float64, device="cuda", generator=g)
    lhs = lsg.apply(op, (2.0 * u - 3.0 * v).contiguous())
    rhs = 2.0 * lsg.apply(op, u) - 3.0 * lsg.apply(op, v)
    assert torch.max(torch.abs(lhs - rhs)).item() < 1e-12
