"""The residual ring of the FP32 AAR (include/lsg.h, lsg_set_aar_form).

The ring's Richardson pass stores only r_k; the Gram and update kernels rebuild
DF_k = (r_k - r_{k-1}) cf and H_k = c r_{k-1} + beta DF_k from two ring slots
with the arithmetic of the x-carrying pass, so the ring and the x-carrying
recurrence (form 2) must give the same iterate, residual and iteration count
bit for bit; the lean form (1) shares the residual trajectory and differs
from them only in how x is accumulated.  Covered: the default cycle (m 7,
p 6), p = 1, a history longer than the cycle, a cycle longer than the
history (p - 1 = m), a stop between extrapolations (the fold), grids whose
size is not a multiple of 4 (the ring does not apply), and the mixed solve,
whose FP64 residual replacements overwrite a ring slot (the column it held is
stored first).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(shape, seed):
    rng = np.random.default_rng(seed)
    b = rng.uniform(-0.5, 0.5, shape[::-1])
    return b - b.mean()


def _solve_forms(lsg, fn, forms=(0, 2, 1)):
    out = {}
    prev = lsg.set_aar_form(0)
    try:
        for f in forms:
            lsg.set_aar_form(f)
            out[f] = fn()
    finally:
        lsg.set_aar_form(prev)
    return out


CASES = [
    ((32, 32, 32), dict(tol=1e-5)),
    ((24, 20, 16), dict(tol=1e-5, m=3, p=1)),
    ((16, 16, 16), dict(tol=1e-5, m=8, p=3, omega=0.8, beta=0.5)),
    ((20, 24, 12), dict(tol=1e-5, m=4, p=5)),
    ((16, 16, 16), dict(max_iter=23, m=5, p=4)),
    ((16, 16, 16), dict(max_iter=17)),
    ((15, 13, 11), dict(tol=1e-5)),  # n % 4 != 0: the lean form runs
    ((15, 16, 12), dict(tol=1e-5)),  # odd nx: the ring passes in the one-column march
    ((16, 12, 20), dict(tol=1e-5, radius=4)),  # generic radius
]


@pytest.mark.parametrize("shape,kw", CASES)
def test_ring_equals_x_carrying_fp32(lsg, shape, kw):
    import torch
    nx = shape[0]
    kw = dict(kw)
    op = lsg.Operator(shape, radius=kw.pop("radius", 6), a=-float(nx * nx), sigma=0.5)
    b = torch.from_numpy(_problem(shape, sum(shape))).to(device="cuda", dtype=torch.float32)
    res = _solve_forms(lsg, lambda: lsg.aar(op, b, **kw))
    (x0, r0), (x2, r2), (x1, r1) = res[0], res[2], res[1]
    assert r0["iters"] == r2["iters"] == r1["iters"]
    assert r0["status"] == r2["status"] == r1["status"]
    assert r0["relres"] == r2["relres"] == r1["relres"]  # the residual trajectory is shared
    if int(np.prod(shape)) % 4:  # no ring: form 0 is the lean form
        assert torch.equal(x0, x1)
        assert ((x2 - x0).norm() / x0.norm()).item() <= 1e-5
    else:
        assert torch.equal(x0, x2), (x0 - x2).abs().max().item()
        assert ((x1 - x0).norm() / x0.norm()).item() <= 1e-5


@pytest.mark.parametrize("n,kw", [(48, dict(tol=1e-10)), (40, dict(tol=1e-10, m=5, p=3, inner_tol=1e-2))])
def test_ring_equals_x_carrying_mixed(lsg, n, kw):
    """Mixed precision: several FP64 replacements, each overwriting the
    residual slot of the extrapolation before it."""
    import torch
    op = lsg.Operator(n, a=-float(n * n), sigma=0.0)
    b = torch.from_numpy(_problem((n, n, n), 7 + n)).cuda()
    res = _solve_forms(lsg, lambda: lsg.aar_mixed(op, b, **kw), forms=(0, 2))
    (x0, r0), (x2, r2) = res[0], res[2]
    assert r0["status"] == 0 and r0["outer_iters"] >= 2
    assert (r0["iters"], r0["outer_iters"]) == (r2["iters"], r2["outer_iters"])
    assert r0["relres"] == r2["relres"]
    assert torch.equal(x0, x2), (x0 - x2).abs().max().item()


def test_ring_form_switch(lsg):
    prev = lsg.set_aar_form(1)
    try:
        assert lsg.set_aar_form(2) == 1
        with pytest.raises(ValueError):
            lsg.set_aar_form(3)
        assert lsg.set_aar_form(0) == 2
    finally:
        lsg.set_aar_form(prev)
