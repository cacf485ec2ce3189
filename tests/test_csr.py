"""General sparse operator path (lsg_aar_csr): AAR on a caller's matrix in
CSR form, Jacobi from the matrix diagonal.  The numpy restatement of AAR.c
with an arbitrary operator (oracle.aar_general) is pinned on CPU against the
C restatement of the stencil solver; on the GPU the CSR solver matches it in
iteration count and solution, reproduces the stencil solver when given the
stencil's own matrix, rejects malformed matrices before any gather, and
serves the drop-in AAR for a user operator bound to its matrix."""
import ctypes as C

import numpy as np
import pytest

scipy_sparse = pytest.importorskip("scipy.sparse")


def stencil_csr(n, radius=6, a=-1.0, sigma=0.0, coeff=None):
    """CSR of the periodic FD operator a * Lap_h + sigma on an n^3 grid (x fastest)."""
    import oracle.oracle as O
    c = O.coefficients(radius) if coeff is None else coeff
    N = n ** 3
    idx = np.arange(N)
    i, j, k = idx % n, (idx // n) % n, idx // (n * n)
    rows, cols, vals = [idx], [idx], [np.full(N, a * 3 * c[0] + sigma)]
    for p in range(1, radius + 1):
        for d in (-p, p):
            for (ii, jj, kk) in (((i + d) % n, j, k), (i, (j + d) % n, k), (i, j, (k + d) % n)):
                rows.append(idx)
                cols.append(ii + n * jj + n * n * kk)
                vals.append(np.full(N, a * c[p]))
    return scipy_sparse.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                                   shape=(N, N))


def variable_coeff_csr(n, seed):
    """7-point -div(k grad) + 0.5 with random conductivities, periodic (SPD, non-constant diagonal)."""
    rng = np.random.default_rng(seed)
    N = n ** 3
    idx = np.arange(N)
    i, j, k = idx % n, (idx // n) % n, idx // (n * n)
    kap = rng.uniform(0.5, 2.0, (3, N))
    rows, cols, vals = [], [], []
    diag = np.full(N, 0.5)
    for ax, (nb) in enumerate((((i + 1) % n) + n * j + n * n * k, i + n * ((j + 1) % n) + n * n * k,
                               i + n * j + n * n * ((k + 1) % n))):
        w = 0.5 * (kap[ax] + kap[ax][nb])
        rows += [idx, nb]
        cols += [nb, idx]
        vals += [-w, -w]
        diag += w
        np.add.at(diag, nb, w)
    rows.append(idx)
    cols.append(idx)
    vals.append(diag)
    return scipy_sparse.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                                   shape=(N, N))


def test_general_restatement_matches_stencil_restatement(oracle):
    n = 10
    A = stencil_csr(n, a=oracle.A_REF)
    rng = np.random.default_rng(0)
    b = rng.uniform(-0.5, 0.5, n ** 3)
    b -= b.mean()
    dinv = 1.0 / A.diagonal()
    xg, rg = oracle.aar_general(lambda v: A @ v, dinv, b, tol=1e-8)
    xs, rs = oracle.solve("aar", b.reshape(n, n, n), tol=1e-8)
    assert rg["iters"] == rs["iters"]
    assert np.linalg.norm(xg - xs.ravel()) <= 1e-9 * np.linalg.norm(xs)


@pytest.mark.gpu
def test_apply_csr_matches_scipy(lsg):
    import torch
    A = variable_coeff_csr(12, 1)
    x = np.random.default_rng(2).standard_normal(A.shape[0])
    y = lsg.apply_csr(lsg.CsrMatrix(A), torch.from_numpy(x).cuda()).cpu().numpy()
    assert np.abs(y - A @ x).max() <= 1e-13 * np.abs(A).max() * np.abs(x).max() * 7


@pytest.mark.gpu
def test_csr_of_the_stencil_reproduces_stencil_aar(lsg, oracle):
    import torch
    n = 16
    A = stencil_csr(n, a=oracle.A_REF)
    b = np.random.default_rng(3).uniform(-0.5, 0.5, n ** 3)
    b -= b.mean()
    bt = torch.from_numpy(b).cuda()
    x, r = lsg.aar_csr(lsg.CsrMatrix(A), bt, tol=1e-8)
    xs, rs = lsg.aar(lsg.Operator(n), bt.reshape(n, n, n), tol=1e-8)
    assert r["status"] == 0 and r["iters"] == rs["iters"]
    assert ((x - xs.reshape(-1)).norm() / xs.norm()).item() <= 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("n,seed,m,p", [(12, 4, 7, 6), (16, 5, 5, 3)])
def test_csr_variable_coefficients(lsg, oracle, n, seed, m, p):
    import torch
    A = variable_coeff_csr(n, seed)
    b = np.random.default_rng(seed).uniform(-0.5, 0.5, n ** 3)
    xo, ro = oracle.aar_general(lambda v: A @ v, 1.0 / A.diagonal(), b, m=m, p=p, tol=1e-10)
    x, r = lsg.aar_csr(lsg.CsrMatrix(A), torch.from_numpy(b).cuda(), m=m, p=p, tol=1e-10)
    assert r["status"] == 0 and ro["converged"]
    assert r["iters"] == ro["iters"]
    x = x.cpu().numpy()
    assert np.linalg.norm(x - xo) <= 1e-8 * np.linalg.norm(xo)
    xd = scipy_sparse.linalg.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x - xd) <= 1e-7 * np.linalg.norm(xd)


@pytest.mark.gpu
def test_malformed_csr_rejected(lsg):
    import torch
    A = variable_coeff_csr(8, 6)
    bad = A.copy()
    bad.indices = bad.indices.copy()
    bad.indices[17] = A.shape[0] + 5  # column out of range
    b = torch.zeros(A.shape[0], dtype=torch.float64, device="cuda")
    with pytest.raises(lsg.CudaLibraryError):
        lsg.aar_csr(lsg.CsrMatrix(bad.indptr, bad.indices, bad.data), b)
    rp = A.indptr.copy()
    rp[5] = rp[6] + 1  # decreasing offsets
    with pytest.raises(lsg.CudaLibraryError):
        lsg.aar_csr(lsg.CsrMatrix(rp, A.indices, A.data), b)


@pytest.mark.gpu
def test_dropin_aar_with_a_user_operator(lsg, oracle):
    """A caller's own Lap_Vec_mult, bound to its matrix, runs through AAR(POISSON*, ...)."""
    n = 12
    A = variable_coeff_csr(n, 7)

    def my_lap(system, a, x, y, comm):  # never called by the library
        raise RuntimeError("host operator callback must not be called")

    cb = lsg.LAP_FN(my_lap)
    lsg.register_operator_csr(cb, A)
    b = np.random.default_rng(8).uniform(-0.5, 0.5, n ** 3)
    x = np.zeros((n, n, n))
    info = lsg.compat_solve("aar", x, b.reshape(n, n, n).copy(), lap=cb, tol=1e-10)
    assert info["status"] == 0 and info["last_status"] == 0
    xo, ro = oracle.aar_general(lambda v: A @ v, 1.0 / A.diagonal(), b, tol=1e-10)
    assert info["iters"] == ro["iters"]
    assert np.linalg.norm(x.ravel() - xo) <= 1e-8 * np.linalg.norm(xo)
    # PGR with a CSR-bound operator is refused, x untouched
    x2 = np.full((n, n, n), 3.0)
    info = lsg.compat_solve("pgr", x2, b.reshape(n, n, n).copy(), lap=cb, tol=1e-10)
    assert info["last_status"] == 6 and (x2 == 3.0).all()
