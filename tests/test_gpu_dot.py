"""lsg_dot: batched conj(x).y kept on the device, against an FP64 torch sum,
for every dtype, batched and not, with sizes that leave partial blocks."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype_name", ["float64", "float32", "complex128", "complex64"])
@pytest.mark.parametrize("shape,batched", [((5, 7, 9), False), ((3, 17, 16, 15), True), ((1, 64, 64, 64), True)])
def test_dot_matches_fp64(lsg, dtype_name, shape, batched):
    import torch
    dt = getattr(torch, dtype_name)
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(shape, dtype=dt, device="cuda", generator=g)
    y = torch.randn(shape, dtype=dt, device="cuda", generator=g)
    got = lsg.dot(x, y, batched=batched)
    hp = torch.complex128 if x.is_complex() else torch.float64
    prod = x.to(hp).conj() * y.to(hp)
    want = prod.reshape(shape[0], -1).sum(1) if batched else prod.sum()
    assert got.shape == want.shape and got.dtype == want.dtype
    scale = (x.to(hp).abs() * y.to(hp).abs()).sum().item()
    assert (got - want).abs().max().item() <= 1e-13 * scale
    # deterministic: the same bits twice
    assert torch.equal(got, lsg.dot(x, y, batched=batched))
