"""Python binding of liblsg (ctypes over the C ABI in include/lsg.h).

Device vectors are torch CUDA tensors shaped ``(nz, ny, nx)`` (x fastest, the
reference layout of MPI_REAL/system.c:82) or flat; PyTorch supplies memory and
streams only — every operation runs in liblsg's own sm_103a kernels.  If the
library cannot be loaded the calls raise; there is no fallback path.

    import lsg
    op = lsg.Operator((256, 256, 256))            # a = -1/(4 pi), FDn = 6, Jacobi
    x, info = lsg.aar(op, b)                       # b: torch.float64 CUDA tensor
    x, info = lsg.aar_mixed(op, b, tol=1e-8)       # FP32 inner / FP64 refinement

The reference's own entry points on host arrays (``AAR(POISSON*, ...)``) are
reachable through ``compat_solve``.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblsg.so")
MAX_RADIUS = 8
MAX_M = 32
A_REF = -1.0 / (4.0 * math.pi)  # operator scale of MPI_REAL/main.c:68

F64, F32, C128, C64 = 0, 1, 2, 3
STATUS = {0: "ok", 1: "not converged", 2: "NaN/Inf detected", 3: "bad argument", 4: "CUDA error",
          5: "timeout", 6: "unsupported", 7: "out of memory", 8: "SVD sweep limit",
          9: "value beyond the double-float stencil range"}


class CudaLibraryError(RuntimeError):
    pass


class _Operator(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("radius", C.c_int), ("coeff", C.c_double * (MAX_RADIUS + 1)),
                ("a", C.c_double), ("sigma", C.c_double), ("precond", C.c_int),
                ("sigma_im", C.c_double)]


class _Params(C.Structure):
    _fields_ = [("omega", C.c_double), ("beta", C.c_double), ("m", C.c_int), ("p", C.c_int),
                ("max_iter", C.c_int), ("tol", C.c_double), ("inner_tol", C.c_double),
                ("max_outer", C.c_int), ("check_every", C.c_int)]


class _Result(C.Structure):
    _fields_ = [("iters", C.c_int), ("relres", C.c_double), ("rhs_norm", C.c_double),
                ("status", C.c_int), ("outer_iters", C.c_int), ("inner_iters", C.c_int),
                ("seconds", C.c_double), ("launches", C.c_longlong), ("svd_fallbacks", C.c_int)]


class _KernelStats(C.Structure):
    _fields_ = [("launches", C.c_longlong * 8), ("ms", C.c_double * 8)]


class _TuneInfo(C.Structure):
    _fields_ = [("tile", C.c_int), ("threads_y", C.c_int), ("rows_per_thread", C.c_int), ("lz", C.c_int),
                ("us_best", C.c_double), ("us_default", C.c_double), ("candidates", C.c_int)]


class _Csr(C.Structure):
    _fields_ = [("n", C.c_int), ("nnz", C.c_longlong), ("row_ptr", C.c_void_p), ("col", C.c_void_p),
                ("val", C.c_void_p), ("precond", C.c_int), ("lanes_per_row", C.c_int)]


class POISSON(C.Structure):
    """Leading fields of MPI_REAL/system.h:26-63 (all the library reads)."""
    _fields_ = [("FDn", C.c_int), ("ssize", C.c_int * 3), ("psize", C.c_int * 3),
                ("np", C.c_int * 3), ("coords", C.c_int * 3), ("rem", C.c_int * 3),
                ("send_neighs", C.c_void_p), ("rec_neighs", C.c_void_p),
                ("send_counts", C.c_void_p), ("rec_counts", C.c_void_p),
                ("send_layers", C.c_int * 6), ("rec_layers", C.c_int * 6),
                ("scounts", C.c_void_p), ("sdispls", C.c_void_p), ("rcounts", C.c_void_p),
                ("rdispls", C.c_void_p), ("n_in", C.c_int), ("n_out", C.c_int),
                ("phi", C.c_void_p), ("rhs", C.c_void_p), ("Lap_phi", C.c_void_p),
                ("solver_tol", C.c_double), ("solver_maxiter", C.c_int), ("m", C.c_int),
                ("p", C.c_int), ("omega", C.c_double), ("beta", C.c_double),
                ("coeff_lap", C.POINTER(C.c_double)), ("comm_laplacian", C.c_long),
                ("cart", C.c_long)]


LAP_FN = C.CFUNCTYPE(None, C.POINTER(POISSON), C.c_double, C.POINTER(C.c_double),
                     C.POINTER(C.c_double), C.c_long)
PRECOND_FN = C.CFUNCTYPE(None, C.c_double, C.POINTER(C.c_double), C.c_int)

_lib = None
_lock = threading.Lock()

EXPORTS = ["lsg_lap_coefficient", "lsg_operator_init", "lsg_params_default", "lsg_apply",
           "lsg_aar", "lsg_pgr", "lsg_pl2r", "lsg_cg", "lsg_aar_mixed", "lsg_pinv_solve",
           "lsg_release_workspaces", "lsg_last_status", "lsg_last_error", "lsg_status_string",
           "lsg_version", "AAR", "PGR", "PL2R", "CG", "lsg_register_operator_callback",
           "lsg_register_precondition_callback", "lsg_set_verbose", "lsg_last_result",
           "lsg_profile", "lsg_profile_read", "lsg_set_compat_mode", "lsg_aar_mixed_c",
           "lsg_pinv_solve_noalloc", "lsg_aar_batched", "lsg_aar_mixed_batched", "lsg_autotune",
           "lsg_set_autotune", "lsg_autotune_save", "lsg_autotune_load", "lsg_gmres",
           "lsg_aar_csr", "lsg_apply_csr", "lsg_register_operator_csr", "lsg_bounds_errors",
           "lsg_set_fp64_arith", "lsg_aar_icc", "lsg_icc_factor", "lsg_cocg", "lsg_set_aar_form", "lsg_dot", "lsg_dot_blocks", "lsg_set_batch_march", "lsg_lgmres"]

KERNEL_CLASSES = ["richardson", "residual", "gram", "update", "small", "cg", "refine", "precond"]


def lib(build_if_missing: bool = True) -> C.CDLL:
    """Loads liblsg.so (building it first if it is absent and nvcc exists)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH) and build_if_missing:
            import importlib.util
            spec = importlib.util.spec_from_file_location("lsg_build", os.path.join(HERE, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        if not os.path.exists(LIB_PATH):
            raise CudaLibraryError(f"{LIB_PATH} missing: build it with linear-solver_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        vp, ip, dp = C.c_void_p, C.c_int, C.c_double
        L.lsg_lap_coefficient.argtypes = [ip, C.POINTER(dp)]
        L.lsg_operator_init.argtypes = [C.POINTER(_Operator), ip, ip, ip, ip, dp, dp, ip]
        L.lsg_params_default.argtypes = [C.POINTER(_Params)]
        L.lsg_params_default.restype = None
        L.lsg_apply.argtypes = [C.POINTER(_Operator), ip, vp, vp, vp]
        for f in ("lsg_aar", "lsg_pgr", "lsg_pl2r", "lsg_cg", "lsg_gmres", "lsg_cocg"):
            getattr(L, f).argtypes = [C.POINTER(_Operator), C.POINTER(_Params), ip, vp, vp,
                                      C.POINTER(_Result), vp]
        L.lsg_aar_mixed.argtypes = [C.POINTER(_Operator), C.POINTER(_Params), vp, vp,
                                    C.POINTER(_Result), vp]
        L.lsg_aar_mixed_c.argtypes = [C.POINTER(_Operator), C.POINTER(_Params), vp, vp,
                                      C.POINTER(_Result), vp]
        L.lsg_pinv_solve.argtypes = [vp, vp, vp, ip, vp]
        L.lsg_aar_csr.argtypes = [C.POINTER(_Csr), C.POINTER(_Params), vp, vp, C.POINTER(_Result), vp]
        L.lsg_apply_csr.argtypes = [C.POINTER(_Csr), vp, vp, vp]
        L.lsg_register_operator_csr.argtypes = [vp, ip, C.c_longlong, C.POINTER(ip), C.POINTER(ip),
                                                C.POINTER(dp)]
        L.lsg_autotune.argtypes = [C.POINTER(_Operator), ip, C.POINTER(_TuneInfo), vp]
        L.lsg_set_autotune.argtypes = [ip]
        L.lsg_set_fp64_arith.argtypes = [ip]
        L.lsg_set_aar_form.argtypes = [ip]
        L.lsg_set_batch_march.argtypes = [ip]
        L.lsg_lgmres.argtypes = [C.POINTER(_Operator), C.POINTER(_Params), ip, ip, vp, vp, C.POINTER(_Result), vp]
        L.lsg_dot_blocks.argtypes = [C.c_longlong]
        L.lsg_dot.argtypes = [ip, ip, C.c_longlong, vp, vp, vp, vp, vp]
        L.lsg_aar_icc.argtypes = [C.POINTER(_Operator), C.POINTER(_Params), C.POINTER(ip), vp, vp,
                                  C.POINTER(_Result), vp]
        L.lsg_icc_factor.argtypes = [C.POINTER(_Operator), C.POINTER(ip), C.POINTER(dp), C.POINTER(dp),
                                     C.POINTER(dp)]
        L.lsg_autotune_save.argtypes = [C.c_char_p]
        L.lsg_autotune_load.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
        L.lsg_bounds_errors.argtypes = [C.POINTER(C.c_longlong)]
        for f in ("lsg_aar_batched", "lsg_aar_mixed_batched"):
            getattr(L, f).argtypes = [C.POINTER(_Operator), ip, C.POINTER(_Params), ip,
                                      C.POINTER(vp), C.POINTER(vp), C.POINTER(_Result), vp]
        L.lsg_last_error.restype = C.c_char_p
        L.lsg_status_string.restype = C.c_char_p
        L.lsg_version.restype = C.c_char_p
        L.lsg_register_operator_callback.argtypes = [vp]
        L.lsg_register_precondition_callback.argtypes = [vp]
        L.lsg_set_verbose.argtypes = [ip]
        L.lsg_set_verbose.restype = None
        L.lsg_last_result.argtypes = [C.POINTER(_Result)]
        L.lsg_last_result.restype = None
        L.AAR.argtypes = [C.POINTER(POISSON), LAP_FN, PRECOND_FN, dp, C.POINTER(dp), C.POINTER(dp),
                          dp, dp, ip, ip, ip, dp, ip, C.c_long]
        L.AAR.restype = None
        for f in ("PGR", "PL2R"):
            getattr(L, f).argtypes = [C.POINTER(POISSON), LAP_FN, PRECOND_FN, dp, C.POINTER(dp),
                                      C.POINTER(dp), dp, ip, ip, ip, dp, ip, C.c_long]
            getattr(L, f).restype = None
        L.CG.argtypes = [C.POINTER(POISSON), LAP_FN, PRECOND_FN, dp, C.POINTER(dp), C.POINTER(dp),
                         ip, dp, ip, C.c_long]
        L.CG.restype = None
        L.lsg_profile.argtypes = [ip]
        L.lsg_profile_read.argtypes = [C.POINTER(_KernelStats)]
        L.lsg_set_compat_mode.argtypes = [ip]
        L.lsg_set_compat_mode.restype = None
        _lib = L
        return L


def exported_symbols():
    return list(EXPORTS)


def _check(rc: int, what: str, allow=(0, 1, 2, 8)):
    if rc not in allow:
        msg = lib().lsg_last_error().decode(errors="replace")
        raise CudaLibraryError(f"{what}: {STATUS.get(rc, rc)}: {msg}")
    return rc


def bounds_errors():
    """Bounds-checked build: the first out-of-range index a stencil march met
    (-1: none).  None for the normal build."""
    v = C.c_longlong(-1)
    rc = lib().lsg_bounds_errors(C.byref(v))
    return None if rc == 6 else v.value


def lap_coefficient(radius: int):
    c = (C.c_double * (MAX_RADIUS + 1))()
    _check(lib().lsg_lap_coefficient(radius, c), "lsg_lap_coefficient", allow=(0,))
    return [c[i] for i in range(radius + 1)]


class Operator:
    """A = a * Lap_h + sigma * I on a periodic (nx, ny, nz) grid, FD half-width `radius`.

    sigma may be complex (the shifted Helmholtz operator of the complex solver)."""

    def __init__(self, n, radius: int = 6, a: float = A_REF, sigma=0.0, precond: bool = True):
        if isinstance(n, int):
            n = (n, n, n)
        self.n = tuple(int(v) for v in n)  # (nx, ny, nz)
        sg = complex(sigma)
        self.radius, self.a, self.precond = int(radius), float(a), bool(precond)
        self.sigma = sg if sg.imag != 0 else sg.real
        self._s = _Operator()
        _check(lib().lsg_operator_init(C.byref(self._s), *self.n, self.radius, self.a, sg.real,
                                       int(self.precond)), "lsg_operator_init", allow=(0,))
        self._s.sigma_im = sg.imag

    @property
    def shape(self):
        return (self.n[2], self.n[1], self.n[0])

    @property
    def numel(self):
        return self.n[0] * self.n[1] * self.n[2]

    @property
    def diag(self):
        return self.a * 3.0 * self._s.coeff[0] + self.sigma

    @property
    def coeff(self):
        return [self._s.coeff[i] for i in range(self.radius + 1)]


def _params(omega=0.6, beta=0.6, m=7, p=6, max_iter=100000, tol=1e-8, inner_tol=3e-4,
            max_outer=50, check_every=0) -> _Params:
    prm = _Params()
    lib().lsg_params_default(C.byref(prm))
    prm.omega, prm.beta, prm.m, prm.p = omega, beta, m, p
    prm.max_iter, prm.tol, prm.inner_tol = max_iter, tol, inner_tol
    prm.max_outer, prm.check_every = max_outer, check_every
    return prm


def _stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _dtype_code(t):
    import torch
    codes = {torch.float64: F64, torch.float32: F32, torch.complex128: C128, torch.complex64: C64}
    if t.dtype in codes:
        return codes[t.dtype]
    raise TypeError(f"unsupported dtype {t.dtype}")


def _check_vec(t, op: Operator, name: str):
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if t.numel() != op.numel:
        raise ValueError(f"{name} has {t.numel()} values, grid has {op.numel}")


def _result(r: _Result) -> dict:
    return dict(iters=r.iters, relres=r.relres, rhs_norm=r.rhs_norm, status=r.status,
                status_name=STATUS.get(r.status, str(r.status)), outer_iters=r.outer_iters,
                inner_iters=r.inner_iters, seconds=r.seconds, launches=r.launches,
                svd_fallbacks=r.svd_fallbacks)


def apply(op: Operator, x, out=None, stream=None):
    """y = A x on the device."""
    import torch
    _check_vec(x, op, "x")
    y = torch.empty_like(x) if out is None else out
    _check(lib().lsg_apply(C.byref(op._s), _dtype_code(x), C.c_void_p(x.data_ptr()),
                           C.c_void_p(y.data_ptr()), _stream_ptr(stream)), "lsg_apply", allow=(0,))
    return y


def _solve(fn: str, op: Operator, b, x0=None, stream=None, **kw):
    import torch
    _check_vec(b, op, "b")
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    _check_vec(x, op, "x0")
    if x.dtype != b.dtype:
        raise TypeError("x0 and b dtypes differ")
    res = _Result()
    prm = _params(**kw)
    rc = getattr(lib(), fn)(C.byref(op._s), C.byref(prm), _dtype_code(b), C.c_void_p(x.data_ptr()),
                            C.c_void_p(b.data_ptr()), C.byref(res), _stream_ptr(stream))
    _check(rc, fn)
    return x, _result(res)


def aar(op, b, x0=None, **kw):
    """Alternating Anderson-Richardson (MPI_REAL/AAR.c:37)."""
    return _solve("lsg_aar", op, b, x0, **kw)


def pgr(op, b, x0=None, **kw):
    """Periodic Galerkin-Richardson (MPI_REAL/PGR.c:35)."""
    return _solve("lsg_pgr", op, b, x0, **kw)


def pl2r(op, b, x0=None, **kw):
    """Periodic L2-Richardson (MPI_REAL/PL2R.c:35)."""
    return _solve("lsg_pl2r", op, b, x0, **kw)


def cg(op, b, x0=None, **kw):
    """Jacobi-preconditioned CG (MPI_REAL/CG.c:33)."""
    return _solve("lsg_cg", op, b, x0, **kw)


def aar_icc(op, b, x0=None, block=(8, 8, 8), stream=None, **kw):
    """AAR with block-Jacobi ICC(0) on (bx, by, bz) boxes, the reference's pc = 1
    (PETSC_REAL/AAR_Real.c:58-61); FP64 vectors."""
    import torch
    _check_vec(b, op, "b")
    if b.dtype != torch.float64:
        raise TypeError("aar_icc: float64 vectors")
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    res = _Result()
    prm = _params(**kw)
    blk = (C.c_int * 3)(*[int(v) for v in block])
    rc = lib().lsg_aar_icc(C.byref(op._s), C.byref(prm), blk, C.c_void_p(x.data_ptr()),
                           C.c_void_p(b.data_ptr()), C.byref(res), _stream_ptr(stream))
    _check(rc, "lsg_aar_icc")
    return x, _result(res)


def icc_factor(op, block=(8, 8, 8)):
    """The block ICC(0) factor on the host: (L (points x 18), d (points), shift)."""
    import numpy as np
    nb = int(block[0]) * int(block[1]) * int(block[2])
    L = np.zeros(nb * 18)
    d = np.zeros(nb)
    sh = C.c_double(0.0)
    blk = (C.c_int * 3)(*[int(v) for v in block])
    dp = C.POINTER(C.c_double)
    _check(lib().lsg_icc_factor(C.byref(op._s), blk, L.ctypes.data_as(dp), d.ctypes.data_as(dp), C.byref(sh)),
           "lsg_icc_factor", allow=(0,))
    return L.reshape(nb, 18), d, sh.value


def lgmres(op, b, x0=None, restart=30, aug=2, stream=None, **kw):
    """LGMRES(restart, aug), the reference's KSPLGMRES comparator
    (PETSC_COMPLEX/main.c:123-147): restart = the whole approximation space,
    restart - aug Krylov vectors plus the last aug error approximations."""
    import torch
    _check_vec(b, op, "b")
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    res = _Result()
    kw = dict(kw)
    kw["m"] = restart
    prm = _params(**kw)
    rc = lib().lsg_lgmres(C.byref(op._s), C.byref(prm), int(aug), _dtype_code(b), C.c_void_p(x.data_ptr()),
                          C.c_void_p(b.data_ptr()), C.byref(res), _stream_ptr(stream))
    _check(rc, "lsg_lgmres")
    return x, _result(res)


def gmres(op, b, x0=None, restart=30, **kw):
    """Restarted GMRES(restart), the reference's PETSc comparator (PETSC_REAL/main.c:84-122)."""
    kw = dict(kw)
    kw["m"] = restart
    return _solve("lsg_gmres", op, b, x0, **kw)


def cocg(op, b, x0=None, **kw):
    """BiCG on the complex-symmetric shifted operator in its COCG form (the
    reference's KSPBICG, PETSC_COMPLEX/main.c:150-175); complex vectors."""
    return _solve("lsg_cocg", op, b, x0, **kw)


SOLVERS = {"aar": aar, "pgr": pgr, "pl2r": pl2r, "cg": cg, "gmres": gmres, "cocg": cocg}


def aar_mixed(op, b, x0=None, stream=None, **kw):
    """FP32 AAR with FP64 residual replacement (include/lsg.h).

    b and x are float64, or complex128 (complex64 inner iteration)."""
    import torch
    if b.dtype not in (torch.float64, torch.complex128):
        raise TypeError("aar_mixed takes float64 or complex128 b / x")
    _check_vec(b, op, "b")
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    res = _Result()
    prm = _params(**kw)
    fn = lib().lsg_aar_mixed if b.dtype == torch.float64 else lib().lsg_aar_mixed_c
    rc = fn(C.byref(op._s), C.byref(prm), C.c_void_p(x.data_ptr()), C.c_void_p(b.data_ptr()),
            C.byref(res), _stream_ptr(stream))
    _check(rc, "lsg_aar_mixed")
    return x, _result(res)


def aar_batched(ops, bs, x0s=None, mixed=False, stream=None, **kw):
    """Batched AAR: solve ops[i] x_i = bs[i] for every i in lockstep.

    Each launch covers all unfinished instances and one extrapolation cycle
    is replayed as a CUDA graph (include/lsg.h, lsg_aar_batched).  bs: CUDA
    tensors of one dtype (float64 / float32 / complex128 / complex64; with
    mixed=True float64 or complex128).  Returns (list of x, list of result dicts).
    """
    import torch
    if len(ops) != len(bs) or not ops:
        raise ValueError("ops and bs must be non-empty lists of equal length")
    dt = bs[0].dtype
    for i, (op, b) in enumerate(zip(ops, bs)):
        _check_vec(b, op, f"bs[{i}]")
        if b.dtype != dt:
            raise TypeError("all right-hand sides must share one dtype")
    if mixed and dt not in (torch.float64, torch.complex128):
        raise TypeError("mixed batched AAR takes float64 or complex128 vectors")
    xs = [torch.zeros_like(b) if x0s is None else x0s[i].clone() for i, b in enumerate(bs)]
    count = len(ops)
    arr = (_Operator * count)(*[op._s for op in ops])
    xp = (C.c_void_p * count)(*[x.data_ptr() for x in xs])
    bp = (C.c_void_p * count)(*[b.data_ptr() for b in bs])
    res = (_Result * count)()
    prm = _params(**kw)
    fn = lib().lsg_aar_mixed_batched if mixed else lib().lsg_aar_batched
    rc = fn(arr, count, C.byref(prm), _dtype_code(bs[0]), xp, bp, res, _stream_ptr(stream))
    _check(rc, "lsg_aar_mixed_batched" if mixed else "lsg_aar_batched")
    return xs, [_result(r) for r in res]


def autotune(op: Operator, dtype, stream=None) -> dict:
    """Times the Richardson pass's launch shapes for op's grid and dtype; caches the fastest.

    dtype: a torch dtype or one of F64 / F32 / C128 / C64."""
    import torch
    code = dtype if isinstance(dtype, int) else {torch.float64: F64, torch.float32: F32,
                                                 torch.complex128: C128, torch.complex64: C64}[dtype]
    info = _TuneInfo()
    _check(lib().lsg_autotune(C.byref(op._s), code, C.byref(info), _stream_ptr(stream)), "lsg_autotune",
           allow=(0,))
    return dict(tile=info.tile, threads_y=info.threads_y, rows_per_thread=info.rows_per_thread, lz=info.lz,
                us_best=info.us_best, us_default=info.us_default, candidates=info.candidates)


def set_autotune(mode: int):
    """0: default launch shapes; 1: cached tuned shapes (default); 2: tune each new grid / batch."""
    _check(lib().lsg_set_autotune(int(mode)), "lsg_set_autotune", allow=(0,))


def set_fp64_arith(mode: int) -> int:
    """Arithmetic of the FP64 stencil passes in the solvers: 0 = double-float
    sums on the FP32 pipe (default; tol < 1e-10 takes FP64 anyway), 1 = FP64
    arithmetic.  Returns the previous mode."""
    return int(lib().lsg_set_fp64_arith(int(mode)))


def dot(x, y, batched: bool = False, stream=None):
    """conj(x) . y on the device (FP64 accumulation, fixed order, no host sync).

    batched: x and y are (B, ...) and the result has one value per leading
    index.  Returns a float64 (real inputs) or complex128 tensor on x's device."""
    import torch
    if x.dtype != y.dtype or x.shape != y.shape or not (x.is_cuda and y.is_cuda):
        raise TypeError("dot: x and y must be CUDA tensors of one dtype and shape")
    x, y = x.contiguous(), y.contiguous()
    count = x.shape[0] if batched else 1
    n = x.numel() // count
    w = 2 if x.is_complex() else 1
    nblk = int(lib().lsg_dot_blocks(n))
    scratch = torch.empty(count * nblk * w, dtype=torch.float64, device=x.device)
    out = torch.empty(count * w, dtype=torch.float64, device=x.device)
    _check(lib().lsg_dot(_dtype_code(x), count, n, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                         C.c_void_p(out.data_ptr()), C.c_void_p(scratch.data_ptr()), _stream_ptr(stream)), "lsg_dot")
    if w == 2:
        out = torch.view_as_complex(out.view(count, 2))
    return out if batched else out.reshape(())


def set_batch_march(paired: bool) -> bool:
    """FP32 batched Richardson passes: paired march (default) or one column per
    lane; identical results.  Returns the previous setting."""
    return bool(lib().lsg_set_batch_march(1 if paired else 0))


def set_aar_form(form: int) -> int:
    """Form of the FP32 AAR's Richardson passes: 0 = residual ring (default
    where it applies), 1 = lean (r', H, DF stored), 2 = x-carrying recurrence.
    All give the same residuals and steps bit for bit.  Returns the previous form."""
    prev = int(lib().lsg_set_aar_form(int(form)))
    if prev < 0:
        raise ValueError(f"AAR form {form} outside 0..2")
    return prev


def autotune_save(path: str):
    _check(lib().lsg_autotune_save(path.encode()), "lsg_autotune_save", allow=(0,))


def autotune_load(path: str) -> int:
    """Adds the tuned shapes of a file written by autotune_save; returns the entries read."""
    n = C.c_int(0)
    _check(lib().lsg_autotune_load(path.encode(), C.byref(n)), "lsg_autotune_load", allow=(0,))
    return n.value


class CsrMatrix:
    """A square sparse matrix on the device in CSR form (int32 offsets and
    indices, float64 values) for lsg_aar_csr / lsg_apply_csr.  Build it from
    a scipy.sparse matrix or from (indptr, indices, data) arrays."""

    def __init__(self, indptr, indices=None, data=None, precond: bool = True, lanes_per_row: int = 0):
        import numpy as np
        import torch
        if indices is None:  # a scipy.sparse matrix
            A = indptr.tocsr()
            indptr, indices, data = A.indptr, A.indices, A.data
        self.indptr = torch.as_tensor(np.asarray(indptr, dtype=np.int32)).cuda()
        self.indices = torch.as_tensor(np.asarray(indices, dtype=np.int32)).cuda()
        self.data = torch.as_tensor(np.asarray(data, dtype=np.float64)).cuda()
        self.n = int(self.indptr.numel()) - 1
        self.precond = bool(precond)
        self._s = _Csr(self.n, int(self.indices.numel()), self.indptr.data_ptr(), self.indices.data_ptr(),
                       self.data.data_ptr(), int(self.precond), int(lanes_per_row))


def aar_csr(A: CsrMatrix, b, x0=None, stream=None, **kw):
    """AAR (MPI_REAL/AAR.c:37-177) with a general sparse operator; b float64 (n,)."""
    import torch
    if b.dtype != torch.float64 or not b.is_cuda or b.numel() != A.n:
        raise ValueError("b must be a float64 CUDA tensor with n values")
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    res = _Result()
    prm = _params(**kw)
    rc = lib().lsg_aar_csr(C.byref(A._s), C.byref(prm), C.c_void_p(x.data_ptr()), C.c_void_p(b.data_ptr()),
                           C.byref(res), _stream_ptr(stream))
    _check(rc, "lsg_aar_csr")
    return x, _result(res)


def apply_csr(A: CsrMatrix, x, stream=None):
    import torch
    y = torch.empty_like(x)
    _check(lib().lsg_apply_csr(C.byref(A._s), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                               _stream_ptr(stream)), "lsg_apply_csr", allow=(0,))
    return y


def register_operator_csr(callback, A_scipy):
    """Bind a ctypes operator callback (a Lap_Vec_mult of the caller's own) to
    the CSR form of its matrix, so the drop-in AAR solves with it on the GPU."""
    import numpy as np
    A = A_scipy.tocsr()
    rp = np.ascontiguousarray(A.indptr, dtype=np.int32)
    ci = np.ascontiguousarray(A.indices, dtype=np.int32)
    va = np.ascontiguousarray(A.data, dtype=np.float64)
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    _check(lib().lsg_register_operator_csr(C.cast(callback, C.c_void_p), A.shape[0], int(A.nnz),
                                           rp.ctypes.data_as(ip), ci.ctypes.data_as(ip),
                                           va.ctypes.data_as(dp)), "lsg_register_operator_csr", allow=(0,))


def pinv_solve(A, b, stream=None):
    """x = pinv(A) b with the reference semantics (MPI_REAL/tools.c:52-105), one warp on the GPU."""
    import torch
    A = A.to(dtype=torch.float64).contiguous()
    b = b.to(dtype=torch.float64).contiguous()
    x = torch.zeros_like(b)
    rc = lib().lsg_pinv_solve(C.c_void_p(A.data_ptr()), C.c_void_p(b.data_ptr()),
                              C.c_void_p(x.data_ptr()), int(b.numel()), _stream_ptr(stream))
    _check(rc, "lsg_pinv_solve", allow=(0, 8))
    return x, rc


def profile(on: bool):
    """Start (clearing totals) or stop per-kernel-class CUDA-event timing."""
    lib().lsg_profile(1 if on else 0)


def profile_read() -> dict:
    """{class: (launches, total_ms)} collected since profile(True)."""
    st = _KernelStats()
    lib().lsg_profile_read(C.byref(st))
    return {KERNEL_CLASSES[i]: (st.launches[i], st.ms[i]) for i in range(8)}


def set_compat_mode(mixed: bool):
    """Drop-in AAR precision: False = FP64 (reference semantics), True = mixed."""
    lib().lsg_set_compat_mode(1 if mixed else 0)


def release_workspaces():
    lib().lsg_release_workspaces()


# ----------------------------------------------------------------------------- drop-in entry points

_keep = []


def _dummy_lap(system, a, x, y, comm):  # never called by the library
    raise RuntimeError("host operator callback must not be called")


def _dummy_pc(diag, r, n):  # never called by the library
    raise RuntimeError("host preconditioner callback must not be called")


def reference_callbacks():
    """ctypes callbacks registered as the reference operator / Jacobi preconditioner.

    They stand for MPI_REAL/system.c's Lap_Vec_mult and Precondition when the
    caller is Python; liblsg recognises them by address and never calls them.
    """
    if not _keep:
        lap, pc = LAP_FN(_dummy_lap), PRECOND_FN(_dummy_pc)
        L = lib()
        _check(L.lsg_register_operator_callback(C.cast(lap, C.c_void_p)), "register", allow=(0,))
        _check(L.lsg_register_precondition_callback(C.cast(pc, C.c_void_p)), "register", allow=(0,))
        _keep.extend([lap, pc])
    return _keep[0], _keep[1]


def make_poisson(n, fdn: int = 6):
    """A POISSON struct for a one-rank run on an (nx, ny, nz) grid (MPI_REAL/main.c:29-54)."""
    if isinstance(n, int):
        n = (n, n, n)
    s = POISSON()
    s.FDn = fdn
    for d in range(3):
        s.ssize[d] = n[d]
        s.psize[d] = n[d]
        s.np[d] = 1
    coeff = (C.c_double * (fdn + 1))(*lap_coefficient(fdn))
    s.coeff_lap = C.cast(coeff, C.POINTER(C.c_double))
    s._coeff_keep = coeff
    return s


def compat_solve(solver: str, x, rhs, *, n=None, fdn=6, a=A_REF, precond=True, omega=0.6,
                 beta=0.6, m=7, p=6, max_iter=100000, tol=1e-8, verbose=False, system=None,
                 lap=None, pc=None):
    """Calls the reference-prototype entry point (AAR/PGR/PL2R/CG) on host numpy arrays.

    x (float64, C-contiguous) is overwritten with the solution, as the
    reference does.  Returns the lsg_result of the call as a dict.
    """
    import numpy as np
    L = lib()
    assert x.dtype == np.float64 and x.flags.c_contiguous
    assert rhs.dtype == np.float64 and rhs.flags.c_contiguous
    if n is None:
        nz, ny, nx = x.shape
        n = (nx, ny, nz)
    s = make_poisson(n, fdn) if system is None else system
    rlap, rpc = reference_callbacks()
    lap = rlap if lap is None else lap
    pc = (rpc if precond else PRECOND_FN()) if pc is None else pc
    L.lsg_set_verbose(1 if verbose else 0)
    dp = C.POINTER(C.c_double)
    xp, bp = x.ctypes.data_as(dp), rhs.ctypes.data_as(dp)
    np_ = int(x.size)
    if solver == "aar":
        L.AAR(C.byref(s), lap, pc, a, xp, bp, omega, beta, m, p, max_iter, tol, np_, 3)
    elif solver == "pgr":
        L.PGR(C.byref(s), lap, pc, a, xp, bp, omega, m, p, max_iter, tol, np_, 3)
    elif solver == "pl2r":
        L.PL2R(C.byref(s), lap, pc, a, xp, bp, omega, m, p, max_iter, tol, np_, 3)
    elif solver == "cg":
        L.CG(C.byref(s), lap, pc, a, xp, bp, max_iter, tol, np_, 3)
    else:
        raise ValueError(solver)
    res = _Result()
    L.lsg_last_result(C.byref(res))
    out = _result(res)
    out["last_status"] = L.lsg_last_status()
    return out


# ----------------------------------------------------------------------------- differentiation

def _solve_for(precision: str, op: Operator, rhs, kw: dict):
    import torch
    cplx = rhs.is_complex() or isinstance(op.sigma, complex)
    hi, lo = (torch.complex128, torch.complex64) if cplx else (torch.float64, torch.float32)
    if precision == "mixed":
        return aar_mixed(op, rhs.to(hi).contiguous(), **kw)
    if precision == "fp64":
        return aar(op, rhs.to(hi).contiguous(), **kw)
    if precision == "fp32":
        return aar(op, rhs.to(lo).contiguous(), **kw)
    raise ValueError(precision)


def _solve_batch_for(precision: str, ops, rhs, kw: dict):
    """Batched solves of ops[i] x_i = rhs[i]; rhs (B, nz, ny, nx); returns (B, ...) and results."""
    import torch
    cplx = rhs.is_complex() or any(isinstance(op.sigma, complex) for op in ops)
    hi, lo = (torch.complex128, torch.complex64) if cplx else (torch.float64, torch.float32)
    if precision not in ("mixed", "fp64", "fp32"):
        raise ValueError(precision)
    dt = lo if precision == "fp32" else hi
    bs = [rhs[i].to(dt).contiguous() for i in range(rhs.shape[0])]
    xs, rs = aar_batched(ops, bs, mixed=(precision == "mixed"), **kw)
    return torch.stack(xs), rs


def _raise_failed(what, infos):
    bad = [(i, r) for i, r in enumerate(infos) if r["status"] != 0]
    if bad:
        i, r = bad[0]
        raise CudaLibraryError(f"{what}: instance {i}: {r['status_name']} ({r})")


class _ShiftedSolve:
    """x = A(sigma)^-1 b with A = a * Lap_h + sigma * I.

    A is symmetric (complex symmetric for complex sigma), so A^H is the same
    stencil with conj(sigma).  Backward is the adjoint solve on the same
    kernels: lambda = A^-H (dL/dx), dL/db = lambda, dL/dsigma = -sum conj(x) lambda
    (real case: -lambda . x).  A leading batch dimension of b (with one sigma
    per instance) runs the forward and adjoint solves as one batched solve.
    """

    @staticmethod
    def build():
        import torch

        def conj_op(op):
            return Operator(op.n, radius=op.radius, a=op.a, sigma=complex(op.sigma).conjugate()
                            if isinstance(op.sigma, complex) else op.sigma, precond=op.precond)

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, b, sigma, grid, radius, a, precision, kw):
                batched = b.dim() == 4
                if torch.is_tensor(sigma):
                    # the shifts are operator coefficients on the host: a CUDA
                    # sigma costs one device-to-host copy here (pass a CPU
                    # tensor or numbers to avoid the synchronisation)
                    raw = sigma.detach().cpu().reshape(-1).tolist()
                elif isinstance(sigma, (list, tuple)):
                    raw = list(sigma)
                else:
                    raw = [sigma]
                svals = [v if isinstance(v, complex) else float(v) for v in raw]
                if batched and len(svals) == 1:
                    svals = svals * b.shape[0]
                ops = [Operator(grid, radius=radius, a=a, sigma=s) for s in svals]
                if batched:
                    x, infos = _solve_batch_for(precision, ops, b.detach(), kw)
                else:
                    x, info = _solve_for(precision, ops[0], b.detach(), kw)
                    infos = [info]
                _raise_failed("forward solve", infos)
                out_dt = b.dtype if not (isinstance(svals[0], complex) and not b.is_complex()) else (
                    torch.complex128 if b.dtype == torch.float64 else torch.complex64)
                x = x.to(out_dt)
                ctx.ops, ctx.precision, ctx.kw, ctx.batched = ops, precision, kw, batched
                ctx.sigma_is_tensor = torch.is_tensor(sigma)
                ctx.sigma_shape = sigma.shape if torch.is_tensor(sigma) else None
                ctx.sigma_dtype = sigma.dtype if torch.is_tensor(sigma) else torch.float64
                ctx.b_dtype = b.dtype
                ctx.save_for_backward(x)
                return x

            @staticmethod
            def backward(ctx, gx):
                (x,) = ctx.saved_tensors
                aops = [conj_op(op) for op in ctx.ops]
                if ctx.batched:
                    lam, infos = _solve_batch_for(ctx.precision, aops, gx.contiguous(), ctx.kw)
                else:
                    lam, info = _solve_for(ctx.precision, aops[0], gx.contiguous(), ctx.kw)
                    infos = [info]
                _raise_failed("adjoint solve", infos)
                lam = lam.to(x.dtype)
                gsig = None
                if ctx.sigma_is_tensor and ctx.needs_input_grad[1]:
                    # dL/dsigma = -x^H lambda, one device reduction per instance
                    g = -dot(x, lam, batched=ctx.batched)
                    if not ctx.sigma_dtype.is_complex:
                        g = g.real
                    nsig = 1
                    for d in ctx.sigma_shape:
                        nsig *= d
                    if g.numel() != nsig:  # one sigma shared by the whole batch
                        g = g.sum()
                    gsig = g.to(ctx.sigma_dtype).reshape(ctx.sigma_shape)
                gb = None
                if ctx.needs_input_grad[0]:
                    gb = lam if ctx.b_dtype.is_complex else lam.real if lam.is_complex() else lam
                    gb = gb.to(ctx.b_dtype)
                return gb, gsig, None, None, None, None, None

        return Fn


_Fn = None


def solve_shifted(b, sigma, *, a=A_REF, radius=6, precision="mixed", **kw):
    """Differentiable x = (a Lap_h + sigma I)^-1 b on the periodic grid of b.

    b: CUDA tensor (nz, ny, nx), or (B, nz, ny, nx) for a batch solved by one
    batched solve; real or complex.  sigma: float / complex or a tensor (0-dim,
    or (B,) for a batch; may require grad).  precision: "mixed" (FP32 /
    complex64 AAR + FP64 residual replacement), "fp64" or "fp32" AAR.
    kw: solver parameters (tol, m, p, omega, beta, ...).
    """
    global _Fn
    if _Fn is None:
        _Fn = _ShiftedSolve.build()
    nz, ny, nx = b.shape[-3:]
    return _Fn.apply(b, sigma, (nx, ny, nz), radius, a, precision, dict(kw))
