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


def test_differentiable_batch_16x128(lsg):
    """16 real solves at 128^3 of -Lap x + sigma x = b (a = -n^2), sigma ~ U[0.1, 10],
    b uniform zero-mean, L = 1/2 ||x - x*||^2 with x* i.i.d. normal.  Forward:
    batched mixed AAR to 1e-9; backward: batched adjoint solve.

    Checks (relative): the FP64 reference gradient (FP64 forward and adjoint
    to 1e-11); central finite differences on sigma with step 1e-4 sigma; 8
    random zero-mean directional derivatives in b.

    The sigma difference quotient (L(s+h) - L(s-h)) / 2h is evaluated without
    subtracting two independently rounded solutions: x(s+h) = x(s-h) - 2h y
    with A(s+h) y = x(s-h) holds exactly, and makes x(s+-h) the exact
    solutions for b - r (r the residual of the x(s-h) solve).  Subtracting two
    separate solves instead is limited by their accuracy: x(s+h) - x(s-h) is
    only ~1e-4 sigma / (4 pi^2 + sigma) of x.  In b the loss is quadratic, so
    the central difference along d equals (A^-1 d) . (x - x*) exactly.
    Both reference solutions are mean-free (b is), so their constant mode,
    which the loss weights by mean(x*) / sigma, is projected out."""
    import time
    import torch
    B, n = 16, 128
    rng = np.random.default_rng(5)
    b = rng.uniform(-0.5, 0.5, (B, n, n, n))
    b -= b.mean(axis=(1, 2, 3), keepdims=True)
    xs = rng.standard_normal((B, n, n, n))
    sig = rng.uniform(0.1, 10.0, B)
    bt, xst, st = (torch.from_numpy(v).cuda() for v in (b, xs, sig))
    a = -float(n * n)

    def dot(u, v):
        return (u * v).reshape(B, -1).sum(1)

    def mean_free(v):
        return v - v.reshape(B, -1).mean(1)[:, None, None, None]

    def grads(prec, tol):
        bb = bt.clone().requires_grad_(True)
        ss = st.clone().requires_grad_(True)
        x = lsg.solve_shifted(bb, ss, a=a, precision=prec, tol=tol, max_iter=30000)
        (0.5 * ((x - xst) ** 2).sum()).backward()
        return bb.grad.detach(), ss.grad.detach(), x.detach()

    t0 = time.time()
    gb, gs, x = grads("mixed", 1e-9)
    t1 = time.time()
    gb64, gs64, x64 = grads("fp64", 1e-11)
    # the mixed forward and adjoint stop at a relative FP64 residual <= 1e-9;
    # the error that leaves in x and in the adjoint is that residual amplified
    # by the slow modes (~1e3 here: 0.9e-6 to 1.3e-6 measured for FP64
    # replacements every 3e-2 and every 3e-4 of FP32 residual reduction)
    assert ((gb - gb64).norm() / gb64.norm()).item() <= 3e-6
    # dL/dsigma = -x . lambda sums N products of both signs: its error follows
    # the solves' error times ||x|| ||lambda||, not |dL/dsigma|, so instances
    # whose sum cancels are compared against a floor of 0.1 x the batch's
    # largest |dL/dsigma| (absolute errors here: 1e-11 .. 1e-9)
    def rel(g, ref):
        scale = torch.maximum(ref.abs(), 0.1 * ref.abs().max())
        return ((g - ref).abs() / scale).max().item()

    assert rel(gs, gs64) <= 1e-5
    with torch.no_grad():
        h = 1e-4 * st
        solve = lambda rhs, s, prec, tol: lsg.solve_shifted(rhs, s, a=a, precision=prec, tol=tol,
                                                             max_iter=30000)
        xm = mean_free(solve(bt, st - h, "mixed", 1e-11))
        y = mean_free(solve(xm, st + h, "fp64", 1e-10))
        fd = -dot(y, xm - h[:, None, None, None] * y - xst)
        err64 = rel(gs64, fd)
        err = rel(gs, fd)
        assert err64 <= 1e-7
        assert err <= 1e-5
        g = torch.Generator(device="cuda").manual_seed(3)
        xr = mean_free(x64)
        werr = 0.0
        for _ in range(8):
            d = mean_free(torch.randn(bt.shape, dtype=torch.float64, device="cuda", generator=g))
            yd = mean_free(solve(d, st, "mixed", 1e-10))
            fdd = dot(yd, xr - xst).sum()
            ad = (gb * d).sum()
            werr = max(werr, abs((ad - fdd) / fdd).item())
        assert werr <= 1e-5
    print(f"16 x 128^3: mixed forward+adjoint {t1 - t0:.2f} s; dL/dsigma vs FD: mixed {err:.1e}, "
          f"fp64 {err64:.1e}; b-directions {werr:.1e}")


def test_batched_literal_central_differences(lsg):
    """The batched forward and adjoint (4 instances at 48^3, sigma ~ U[0.1, 10],
    FP64 to 1e-13) against literal two-solve central differences: one batched
    solve at sigma + h and one at sigma - h (h = 1e-4 sigma; the instances are
    independent, so both batches give every dL/dsigma_i at once), and 4 random
    directions d in b, (L(b + eps d) - L(b - eps d)) / 2 eps.  The loss
    differences use L(+) - L(-) = 1/2 (x+ - x-) . (x+ + x- - 2 x*); agreement
    1e-5 relative."""
    import torch
    B, n = 4, 48
    rng = np.random.default_rng(21)
    b = rng.uniform(-0.5, 0.5, (B, n, n, n))
    b -= b.mean(axis=(1, 2, 3), keepdims=True)
    bt = torch.from_numpy(b).cuda()
    xst = torch.from_numpy(rng.standard_normal((B, n, n, n))).cuda()
    st = torch.from_numpy(rng.uniform(0.1, 10.0, B)).cuda()
    a = -float(n * n)
    solve = lambda rhs, s: lsg.solve_shifted(rhs, s, a=a, precision="fp64", tol=1e-13, max_iter=50000)
    bb = bt.clone().requires_grad_(True)
    ss = st.clone().requires_grad_(True)
    (0.5 * ((solve(bb, ss) - xst) ** 2).sum()).backward()
    gb, gs = bb.grad.detach(), ss.grad.detach()

    def dloss(xp, xm):  # per instance
        return 0.5 * ((xp - xm) * (xp + xm - 2 * xst)).reshape(B, -1).sum(1)

    with torch.no_grad():
        h = 1e-4 * st
        fd = dloss(solve(bt, st + h), solve(bt, st - h)) / (2 * h)
        assert ((gs - fd).abs() / fd.abs()).max().item() <= 1e-5, (gs, fd)
        g = torch.Generator(device="cuda").manual_seed(8)
        for _ in range(4):
            d = torch.randn(bt.shape, dtype=torch.float64, device="cuda", generator=g)
            eps = 1e-3 * bt.norm().item() / d.norm().item()
            fdd = dloss(solve(bt + eps * d, st), solve(bt - eps * d, st)).sum() / (2 * eps)
            ad = (gb * d).sum()
            assert abs(((ad - fdd) / fdd).item()) <= 1e-5


def test_gradcheck_complex_8cube(lsg):
    """Complex b and sigma: lambda = A^-H g uses the stencil with conj(sigma) and
    dL/dsigma = -sum conj(x) lambda, checked against torch's conjugate-Wirtinger
    convention by gradcheck."""
    import torch
    n = 8
    rng = np.random.default_rng(11)
    b = torch.from_numpy(rng.uniform(-0.5, 0.5, (n, n, n)) + 1j * rng.uniform(-0.5, 0.5, (n, n, n)))
    b = b.cuda().requires_grad_(True)
    s = torch.tensor(3.0 + 20.0j, dtype=torch.complex128, requires_grad=True)
    f = lambda bb, ss: lsg.solve_shifted(bb, ss, a=-n * n, precision="fp64", tol=1e-13)
    assert torch.autograd.gradcheck(f, (b, s), eps=1e-6, atol=1e-8, rtol=1e-6)


def test_batched_gradient_equals_single(lsg):
    import torch
    B, n = 3, 16
    rng = np.random.default_rng(12)
    b = rng.uniform(-0.5, 0.5, (B, n, n, n))
    xs = torch.from_numpy(rng.standard_normal((B, n, n, n))).cuda()
    sig = torch.tensor([0.5, 3.0, 9.0], dtype=torch.float64, device="cuda")
    bb = torch.from_numpy(b).cuda().requires_grad_(True)
    ss = sig.clone().requires_grad_(True)
    x = lsg.solve_shifted(bb, ss, a=-n * n, precision="fp64", tol=1e-12)
    (0.5 * ((x - xs) ** 2).sum()).backward()
    for i in range(B):
        b1 = torch.from_numpy(b[i]).cuda().requires_grad_(True)
        s1 = sig[i].clone().requires_grad_(True)
        x1 = lsg.solve_shifted(b1, s1, a=-n * n, precision="fp64", tol=1e-12)
        (0.5 * ((x1 - xs[i]) ** 2).sum()).backward()
        assert ((bb.grad[i] - b1.grad).norm() / b1.grad.norm()).item() <= 1e-9
        assert ss.grad[i].item() == pytest.approx(s1.grad.item(), rel=1e-9)
