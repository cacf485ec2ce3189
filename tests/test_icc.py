"""Block-Jacobi ICC(0) (the reference's pc = 1, PETSC_REAL/AAR_Real.c:58-61) on
the CPU: the library's host factor equals the oracle's restatement bit for
bit, and the restated preconditioned AAR needs fewer iterations than Jacobi.

Parity is unpinned by the reference: PETSc 3.11.3 (PCICC) is absent, so the
oracle restates the published incomplete-Cholesky algorithm (zero fill,
natural order) on the same box partition."""
import numpy as np
import pytest


@pytest.mark.parametrize("block,radius,sigma", [((8, 8, 8), 6, 0.0), ((4, 6, 5), 6, 0.3),
                                                ((16, 16, 8), 6, 0.0), ((5, 5, 5), 3, 0.0)])
def test_factor_matches_restatement(lsg, oracle, block, radius, sigma):
    op = lsg.Operator((16, 16, 16), radius=radius, sigma=sigma)
    L, d, shift = lsg.icc_factor(op, block)
    Lo, do, so = oracle.icc0_factor_shifted(block, oracle.stencil_weights(radius, sigma=sigma), radius)
    assert shift == so
    assert np.array_equal(L, Lo) and np.array_equal(d, do)
    assert (d > 0).all()


def test_factor_rejects_bad_box(lsg):
    with pytest.raises(lsg.CudaLibraryError):
        lsg.icc_factor(lsg.Operator(16), (32, 32, 32))  # 32768 points > 4096


def test_icc_aar_restatement_cuts_iterations(oracle):
    """AAR.c with f = M^-1 r: 186 Jacobi iterations -> 78 with 8^3 boxes (32^3, uniform rhs)."""
    import workloads
    n = 32
    b = workloads.uniform_rhs(n, 0)
    w = oracle.stencil_weights()
    mv = lambda v: oracle.apply(v.reshape(n, n, n)).ravel()
    dinv = np.full(n ** 3, 1.0 / w[0])
    _, rj = oracle.aar_general(mv, dinv, b)
    L, d, _ = oracle.icc0_factor_shifted((8, 8, 8), w)
    pc = lambda r: oracle.icc0_apply(r.reshape(n, n, n), (n, n, n), (8, 8, 8), L, d).ravel()
    x, ri = oracle.aar_general(mv, dinv, b, precond=pc)
    assert rj["converged"] and ri["converged"]
    assert ri["iters"] < 0.5 * rj["iters"], (ri, rj)
    res = np.linalg.norm(b.ravel() - mv(x)) / np.linalg.norm(b)
    assert res <= 1e-8


def test_icc_apply_is_inverse_of_factor(oracle):
    """(L D L^T) f = r on every box for the restated apply (the factor's own matrix)."""
    n, blk = 8, (4, 4, 4)
    w = oracle.stencil_weights()
    L, d, _ = oracle.icc0_factor_shifted(blk, w)
    rng = np.random.default_rng(2)
    r = rng.standard_normal((n, n, n))
    f = oracle.icc0_apply(r, (n, n, n), blk, L, d)
    nb = 64
    Lm = np.eye(nb)
    st = (1, 4, 16)
    for i in range(nb):
        c = (i % 4, (i // 4) % 4, i // 16)
        for a in range(3):
            for p in range(1, 7):
                if c[a] >= p:
                    Lm[i, i - p * st[a]] = L[i, 6 * a + p - 1]
    M = Lm @ np.diag(d) @ Lm.T
    fb = f.reshape(2, 4, 2, 4, 2, 4).transpose(0, 2, 4, 1, 3, 5).reshape(-1, nb)
    rb = r.reshape(2, 4, 2, 4, 2, 4).transpose(0, 2, 4, 1, 3, 5).reshape(-1, nb)
    assert np.allclose(fb @ M.T, rb, rtol=0, atol=1e-12 * np.abs(rb).max())
