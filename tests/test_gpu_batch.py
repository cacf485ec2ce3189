"""Batched AAR (one launch per pass over every instance, the extrapolation
cycle replayed as a CUDA graph): each instance against its own single solve
(same iteration count, same solution up to reduction order) and against the
exact FFT solve; mixed precision (FP32 / complex64 inner iteration with FP64 /
complex128 residual replacement); the 48-instance complex shifted-Helmholtz
workload (sides 32..160, sigma_r ~ U[0,50], sigma_i ~ U[1,50]).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _real_problem(n, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    b = rng.uniform(-0.5, 0.5, (nz, ny, nx))
    return b - b.mean()


def _cplx_problem(n, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.5, 0.5, (n, n, n)) + 1j * rng.uniform(-0.5, 0.5, (n, n, n))


def _cuda(x, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to(device="cuda", dtype=dtype)


GRIDS = [16, (20, 18, 12), 24, (12, 16, 20)]


@pytest.mark.parametrize("dtype_name", ["float64", "float32"])
def test_batched_real_matches_single(lsg, dtype_name):
    import torch
    dt = getattr(torch, dtype_name)
    ops, bs = [], []
    for k, n in enumerate(GRIDS):
        b = _real_problem(n, 10 + k)
        nz, ny, nx = b.shape
        ops.append(lsg.Operator((nx, ny, nz), a=-float(nx * nx), sigma=[0.0, 2.0, 0.5, 7.0][k]))
        bs.append(_cuda(b, dt))
    tol = 1e-8 if dt == torch.float64 else 1e-5
    xs, rs = lsg.aar_batched(ops, bs, tol=tol)
    for op, b, x, r in zip(ops, bs, xs, rs):
        xs1, r1 = lsg.aar(op, b, tol=tol)
        assert r["status"] == 0 and r1["status"] == 0
        assert r["iters"] == r1["iters"]
        assert r["relres"] == pytest.approx(r1["relres"], rel=1e-3 if dt == torch.float64 else 2e-2)
        rel = ((x - xs1).norm() / xs1.norm()).item()
        assert rel <= (1e-9 if dt == torch.float64 else 1e-4)


@pytest.mark.parametrize("dtype_name", ["float64", "float32"])
def test_batched_p1_and_max_iter(lsg, dtype_name):
    """p = 1 (iteration 1 is the only Richardson one) and max_iter stops.  In
    FP32 the Richardson passes leave x out, so a stop between extrapolations
    (17, 23) folds the cycle's steps into x, and p = 1 rotates the residual
    buffers differently; each instance must match its single solve."""
    import torch
    dt = getattr(torch, dtype_name)
    ops = [lsg.Operator(n, a=-float(n * n), sigma=1.0) for n in (12, 16)]
    bs = [_cuda(_real_problem(n, 3 + n), dt) for n in (12, 16)]
    for kw in (dict(p=1, m=3), dict(max_iter=17), dict(max_iter=23, m=5, p=4), dict(max_iter=18)):
        xs, rs = lsg.aar_batched(ops, bs, **kw)
        for op, b, x, r in zip(ops, bs, xs, rs):
            x1, r1 = lsg.aar(op, b, **kw)
            assert r["iters"] == r1["iters"] and r["status"] == r1["status"]
            assert ((x - x1).norm() / x1.norm()).item() <= (1e-9 if dt == torch.float64 else 1e-5)


def test_batched_generic_radius(lsg, oracle):
    import torch
    ops, bs, bn = [], [], []
    for k, (n, rad) in enumerate([(16, 4), (12, 4), (20, 4)]):
        b = _real_problem(n, 40 + k)
        ops.append(lsg.Operator(n, radius=rad, a=-float(n * n), sigma=3.0))
        bs.append(_cuda(b, torch.float64))
        bn.append(b)
    xs, rs = lsg.aar_batched(ops, bs, tol=1e-10)
    for op, b, x, r in zip(ops, bn, xs, rs):
        assert r["status"] == 0
        xf = oracle.fft_solve(b, radius=op.radius, a=op.a, sigma=3.0)
        assert np.linalg.norm(x.cpu().numpy() - xf) <= 1e-7 * np.linalg.norm(xf)


@pytest.mark.parametrize("dtype_name", ["complex128", "complex64"])
def test_batched_complex_matches_single(lsg, dtype_name):
    import torch
    dt = getattr(torch, dtype_name)
    sig = [20 + 15j, 3.5 + 40j, 0.5 + 2j]
    ns = [16, 24, 12]
    ops = [lsg.Operator(n, a=-float(n * n), sigma=s) for n, s in zip(ns, sig)]
    bs = [_cuda(_cplx_problem(n, 7 * n), dt) for n in ns]
    tol = 1e-8 if dt == torch.complex128 else 1e-5
    xs, rs = lsg.aar_batched(ops, bs, tol=tol)
    for op, b, x, r in zip(ops, bs, xs, rs):
        x1, r1 = lsg.aar(op, b, tol=tol)
        assert r["status"] == 0
        assert r["iters"] == r1["iters"]
        assert ((x - x1).norm() / x1.norm()).item() <= (1e-9 if dt == torch.complex128 else 1e-4)


def test_batched_mixed_real(lsg, oracle):
    import torch
    ns = [32, 24, 40, 16]
    sig = [0.0, 5.0, 0.3, 40.0]
    ops = [lsg.Operator(n, a=-float(n * n), sigma=s) for n, s in zip(ns, sig)]
    bn = [_real_problem(n, 90 + n) for n in ns]
    bs = [_cuda(b, torch.float64) for b in bn]
    xs, rs = lsg.aar_batched(ops, bs, mixed=True, tol=1e-10)
    for op, b, x, r, s in zip(ops, bn, xs, rs, sig):
        assert r["status"] == 0 and r["relres"] <= 1e-10
        bt = _cuda(b, torch.float64)
        true = ((bt - lsg.apply(op, x)).norm() / bt.norm()).item()
        assert true <= 1e-10 * 1.01
        x1, r1 = lsg.aar_mixed(op, bt, tol=1e-10)
        assert abs(r["iters"] - r1["iters"]) <= 4 * op_p()
        xf = oracle.fft_solve(b, a=op.a, sigma=s)
        lam = np.abs(oracle.symbol(b.shape, a=op.a) + s)
        lam = lam[lam > 1e-12 * lam.max()]
        kappa = lam.max() / lam.min()
        xn = x.cpu().numpy()
        if s == 0.0:  # Poisson: solutions are defined up to the constant (nullspace) mode
            xn = xn - xn.mean()
        assert np.linalg.norm(xn - xf) <= kappa * 1e-10 * np.linalg.norm(xf)


def op_p():
    return 6


def _helmholtz_batch(count, seed, sides=(32, 48, 64, 96, 128, 160)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice(sides))
        sig = complex(rng.uniform(0.0, 50.0), rng.uniform(1.0, 50.0))
        b = rng.uniform(-0.5, 0.5, (n, n, n)) + 1j * rng.uniform(-0.5, 0.5, (n, n, n))
        out.append((n, sig, b))
    return out


def _check_helmholtz(lsg, oracle, batch, tol):
    import torch
    ops = [lsg.Operator(n, a=-float(n * n), sigma=s) for n, s, _ in batch]
    bs = [_cuda(b, torch.complex128) for _, _, b in batch]
    xs, rs = lsg.aar_batched(ops, bs, mixed=True, tol=tol)
    worst = 0.0
    for (n, s, b), op, x, r in zip(batch, ops, xs, rs):
        assert r["status"] == 0 and r["relres"] <= tol
        xf = oracle.fft_solve(b, a=op.a, sigma=s)
        lam = np.abs(oracle.symbol(b.shape, a=op.a) + s)
        kappa = lam.max() / lam.min()
        err = np.linalg.norm(x.cpu().numpy() - xf) / np.linalg.norm(xf)
        assert err <= kappa * tol
        worst = max(worst, err)
    return rs, worst


def test_batched_mixed_complex_small(lsg, oracle):
    batch = _helmholtz_batch(6, 5, sides=(12, 16, 20, 24, 32))
    _check_helmholtz(lsg, oracle, batch, 1e-8)


def test_batched_helmholtz_48(lsg, oracle):
    """48 complex solves, sides drawn from {32, 48, 64, 96, 128, 160}, complex64
    inner iteration with complex128 residual replacement, tol 1e-8."""
    batch = _helmholtz_batch(48, 2024)
    rs, worst = _check_helmholtz(lsg, oracle, batch, 1e-8)
    print(f"48 Helmholtz solves: max error vs FFT {worst:.2e}, "
          f"iterations {min(r['iters'] for r in rs)}..{max(r['iters'] for r in rs)}, "
          f"{rs[0]['seconds']:.3f} s, {rs[0]['launches']} launches")


@pytest.mark.parametrize("mixed", [False, True])
def test_batched_paired_march_bitwise(lsg, mixed):
    """FP32 batches: the paired march of the Richardson passes (two columns
    per lane, 64-wide tiles) against the one-column march, bit for bit, on
    uneven grids (even nx), including a stop between extrapolations and
    p - 1 > m (the x-carrying pass)."""
    import torch
    shapes = [(16, 16, 16), (34, 20, 12), (24, 30, 18), (66, 10, 9)]
    ops = [lsg.Operator(sh, a=-float(sh[0] ** 2), sigma=s) for sh, s in zip(shapes, [0.0, 3.0, 0.5, 9.0])]
    dt = torch.float64 if mixed else torch.float32
    bs = [_cuda(_real_problem(sh, 50 + k), dt) for k, sh in enumerate(shapes)]
    kws = [dict(tol=1e-9)] if mixed else [dict(tol=1e-5), dict(max_iter=23), dict(tol=1e-5, m=2, p=5)]
    for kw in kws:
        prev = lsg.set_batch_march(True)
        try:
            xp, rp = lsg.aar_batched(ops, bs, mixed=mixed, **kw)
            lsg.set_batch_march(False)
            x1, r1 = lsg.aar_batched(ops, bs, mixed=mixed, **kw)
        finally:
            lsg.set_batch_march(prev)
        for a, b, ra, rb in zip(xp, x1, rp, r1):
            assert ra["iters"] == rb["iters"] and ra["status"] == rb["status"]
            assert torch.equal(a, b)
