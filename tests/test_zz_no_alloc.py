"""lsg_pinv_solve_noalloc: the m x m pseudo-inverse solve that allocates nothing.

Callers that cannot call cudaMalloc (device memory owned by an external pool
or capped per client, or a loop that cannot pay an allocation per call) use
this variant; its only scratch, the kernel's status word, sits in a static
device array inside liblsg.  Checked through the C ABI against the allocating
entry point lsg_pinv_solve on the same inputs, twice in a row, to the
tolerance the other pseudo-inverse tests use.  Kept in its own file so that
pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    rng = np.random.default_rng(21)
    F = np.zeros((300, 7))
    F[:, :5] = rng.standard_normal((300, 5))  # rank-deficient Gram (first Anderson step)
    yield F.T @ F, rng.standard_normal(7)
    yield rng.standard_normal((7, 7)), rng.standard_normal(7)  # non-symmetric (PGR)
    G = rng.standard_normal((400, 32))
    yield G.T @ G, rng.standard_normal(32)  # the largest supported m
    yield np.array([[2.5]]), np.array([1.5])


def _solve(L, name, A, b):
    import torch
    x = torch.zeros_like(b)
    rc = getattr(L, name)(C.c_void_p(A.data_ptr()), C.c_void_p(b.data_ptr()),
                          C.c_void_p(x.data_ptr()), int(b.numel()), None)
    torch.cuda.synchronize()
    return rc, x.cpu().numpy()


def test_noalloc_pinv_matches_allocating_entry_point(lsg):
    import torch
    L = lsg.lib()
    L.lsg_pinv_solve_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.lsg_pinv_solve.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    for A, b in _cases():
        At = torch.from_numpy(np.ascontiguousarray(A)).cuda()
        bt = torch.from_numpy(np.ascontiguousarray(b)).cuda()
        rc0, x0 = _solve(L, "lsg_pinv_solve", At, bt)
        assert rc0 == 0
        for _ in range(2):  # two calls in a row share the static scratch
            rc, x = _solve(L, "lsg_pinv_solve_noalloc", At, bt)
            assert rc == 0
            assert np.allclose(x, x0, rtol=1e-8, atol=1e-10 * np.abs(x0).max())


def test_noalloc_pinv_rejects_sizes_beyond_maximum(lsg):
    import torch
    L = lsg.lib()
    L.lsg_pinv_solve_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.lsg_last_error.restype = C.c_char_p
    A = torch.zeros((33, 33), dtype=torch.float64, device="cuda")
    b = torch.zeros(33, dtype=torch.float64, device="cuda")
    rc, _ = _solve(L, "lsg_pinv_solve_noalloc", A, b)
    assert rc == 3
    assert b"outside 1..32" in L.lsg_last_error()
