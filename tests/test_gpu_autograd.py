"""Differentiable shifted solve: the adjoint-solve backward against
torch.autograd.gradcheck, central finite differences (step 1e-4 sigma) on
sigma and on 8 random directions in b, and an FP64-reference gradient.

L = 1/2 ||x - x*||^2 is dominated by ||x*||^2, so the finite differences are
evaluated in the algebraically exact form
L(p+) - L(p-) = 1/2 (x+ - x-) . (x+ + x- - 2 x*), which avoids the
cancellation of subtracting two nearly equal losses.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(n, seed):
    import torch
    rng = np.random.default_rng(seed)
    b = rng.uniform(-0.5, 0.5, n ** 3)
    b -= b.mean()
    xs = rng.standard_normal(n ** 3)
    t = lambda v: torch.from_numpy(v.reshape(n, n, n)).cuda()
    return t(b), t(xs), float(rng.uniform(0.1, 10.0))


def test_gradcheck_fp64_8cube(lsg):
    import torch
    n = 8
    b, _, sig = _problem(n, 1)
    b.requires_grad_(True)
    s = torch.tensor(sig, dtype=torch.float64, requires_grad=True)
    f = lambda bb, ss: lsg.solve_shifted(bb, ss, a=-n * n, precision="fp64", tol=1e-13)
    assert torch.autograd.gradcheck(f, (b, s), eps=1e-6, atol=1e-8, rtol=1e-6)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 1e-14)])
def test_finite_differences_and_fp64_reference(lsg, precision, tol):
    """32^3, a = -n^2 (-Lap_h / h^2 on the unit cube); relative agreement 1e-5.

    x+ - x- is ~1e-5 |x| for the sigma step, so the solves must be accurate to
    well below 1e-10 (cond(A) ~ 4e2 here): hence tol 1e-13 / 1e-14."""
    import torch
    n = 32
    b, xstar, sig = _problem(n, 2)
    a = -float(n * n)
    solve = lambda bb, ss: lsg.solve_shifted(bb, ss, a=a, precision=precision, tol=tol)

    def dloss(xp, xm):  # L(x+) - L(x-)
        return 0.5 * ((xp - xm) * (xp + xm - 2 * xstar)).sum().item()

    bb = b.clone().requires_grad_(True)
    ss = torch.tensor(sig, dtype=torch.float64, requires_grad=True)
    (0.5 * ((solve(bb, ss) - xstar) ** 2).sum()).backward()
    gb, gs = bb.grad.detach(), ss.grad.item()
    with torch.no_grad():
        h = 1e-4 * sig
        fd = dloss(solve(b, sig + h), solve(b, sig - h)) / (2 * h)
        assert gs == pytest.approx(fd, rel=1e-5)
        g = torch.Generator(device="cuda").manual_seed(3)
        for _ in range(8):
            d = torch.randn(b.shape, dtype=torch.float64, device="cuda", generator=g)
            eps = 1e-3 * b.norm().item() / d.norm().item()
            fdd = dloss(solve(b + eps * d, sig), solve(b - eps * d, sig)) / (2 * eps)
            assert (gb * d).sum().item() == pytest.approx(fdd, rel=1e-5)
    # FP64 reference gradient (tight FP64 solves)
    bb2 = b.clone().requires_grad_(True)
    ss2 = torch.tensor(sig, dtype=torch.float64, requires_grad=True)
    x2 = lsg.solve_shifted(bb2, ss2, a=a, precision="fp64", tol=1e-13)
    (0.5 * ((x2 - xstar) ** 2).sum()).backward()
    assert (gb - bb2.grad).norm().item() <= 1e-6 * bb2.grad.norm().item()
    assert gs == pytest.approx(ss2.grad.item(), rel=1e-6)


def test_fp32_gradient_close_to_fp64(lsg):
    """FP32 forward and adjoint: gradient within FP32 solve accuracy of the FP64 one."""
    import torch
    n = 24
    b, xstar, sig = _problem(n, 4)
    a = -float(n * n)
    out = {}
    for prec, tol in (("fp32", 1e-6), ("fp64", 1e-12)):
        bb = b.clone().requires_grad_(True)
        ss = torch.tensor(sig, dtype=torch.float64, requires_grad=True)
        x = lsg.solve_shifted(bb.float() if prec == "fp32" else bb, ss, a=a, precision=prec, tol=tol)
        (0.5 * ((x.double() - xstar) ** 2).sum()).backward()
        out[prec] = (bb.grad.clone(), ss.grad.item())
    assert (out["fp32"][0] - out["fp64"][0]).norm().item() <= 1e-4 * out["fp64"][0].norm().item()
    assert out["fp32"][1] == pytest.approx(out["fp64"][1], rel=1e-3)
