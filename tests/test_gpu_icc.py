"""Block-Jacobi ICC(0) AAR on the GPU (lsg_aar_icc, the reference's pc = 1)
against the oracle's restatement (oracle.aar_general with the block ICC(0)
preconditioner on the same boxes): identical iteration counts and solutions,
in FP64 arithmetic and in the default double-float stencil arithmetic.
Boxes whose factor fits in shared memory (up to ~1000 points) take the
staged kernel that solves four boxes per CTA; 16 x 16 x 8 boxes the
one-box-per-CTA kernel."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_icc(oracle, b, shape, block, radius=6, sigma=0.0, **kw):
    nz, ny, nx = shape
    w = oracle.stencil_weights(radius, sigma=sigma)
    L, d, _ = oracle.icc0_factor_shifted(block, w, radius)
    mv = lambda v: oracle.apply(v.reshape(shape), radius=radius, sigma=sigma).ravel()
    pc = lambda r: oracle.icc0_apply(r.reshape(shape), shape, block, L, d, radius).ravel()
    x, r = oracle.aar_general(mv, np.ones(nx * ny * nz), b, precond=pc, **kw)
    return x.reshape(shape), r


@pytest.mark.parametrize("mode", [1, 0])
@pytest.mark.parametrize("n,block,radius,sigma", [((16, 16, 16), (8, 8, 8), 6, 0.0),
                                                  ((24, 16, 20), (4, 8, 5), 6, 0.0),
                                                  ((16, 16, 16), (8, 4, 8), 3, 0.4),
                                                  ((32, 32, 16), (16, 16, 8), 6, 0.0)])
def test_icc_matches_restatement(lsg, oracle, mode, n, block, radius, sigma):
    import torch
    import workloads
    prev = lsg.set_fp64_arith(mode)
    try:
        nx, ny, nz = n
        rng = np.random.default_rng(7)
        b = rng.uniform(-0.5, 0.5, (nz, ny, nx))
        b -= b.mean()
        xo, ro = _oracle_icc(oracle, b, (nz, ny, nx), block, radius, sigma)
        op = lsg.Operator(n, radius=radius, sigma=sigma)
        x, r = lsg.aar_icc(op, torch.from_numpy(b).cuda(), block=block)
    finally:
        lsg.set_fp64_arith(prev)
    assert r["status"] == 0 and ro["converged"]
    assert r["iters"] == ro["iters"], (r, ro)
    xg = x.cpu().numpy()
    xg, xo = xg - xg.mean(), xo - xo.mean()
    assert np.linalg.norm(xg - xo) / np.linalg.norm(xo) < 1e-7
    del workloads


def test_icc_fewer_iterations_than_jacobi(lsg):
    import torch
    import workloads
    n = 64
    b = torch.from_numpy(workloads.uniform_rhs(n, 2)).cuda()
    op = lsg.Operator(n)
    _, rj = lsg.aar(op, b)
    x, ri = lsg.aar_icc(op, b, block=(8, 8, 8))
    assert rj["status"] == 0 and ri["status"] == 0
    assert ri["iters"] < 0.6 * rj["iters"], (ri, rj)
    true = ((b - lsg.apply(op, x)).norm() / b.norm()).item()
    assert true <= 1e-8 * 1.01


def test_icc_bad_box(lsg):
    import torch
    b = torch.zeros((16, 16, 16), dtype=torch.float64, device="cuda")
    with pytest.raises(lsg.CudaLibraryError, match="divide"):
        lsg.aar_icc(lsg.Operator(16), b, block=(6, 8, 8))
