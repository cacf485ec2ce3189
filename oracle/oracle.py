"""ctypes loader for the CPU checkers — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module.  The product (``liblsg.so`` and its Python binding) never
does.

Two libraries are wrapped:

* ``_build/liblsg_oracle.so`` — the project's C restatement of the reference
  solvers (``lsg_oracle.c``); builds anywhere with gcc.
* ``_ref/libref_mpi_real.so`` — the UNMODIFIED reference sources
  (YaphetS-jx/Linear-Solver ``MPI_REAL``) compiled here by ``make ref`` against
  a one-rank MPI shim, driven through ``ref_harness.c``.  Present only where
  the reference checkout exists; used to pin the restatement.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liblsg_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_mpi_real.so")
MAXR = 16

SOLVERS = {"aar": 0, "pgr": 1, "pl2r": 2, "cg": 3}
A_REF = -1.0 / (4.0 * math.pi)  # operator scale the reference driver passes (MPI_REAL/main.c:68)


class OpStruct(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("radius", C.c_int), ("coeff", C.c_double * (MAXR + 1)),
                ("a", C.c_double), ("sigma", C.c_double)]


class ResultStruct(C.Structure):
    _fields_ = [("iters", C.c_int), ("relres", C.c_double), ("rhs_norm", C.c_double),
                ("converged", C.c_int), ("status", C.c_int), ("seconds", C.c_double)]


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def reference_dir() -> str:
    """Where the reference's MPI_REAL sources are: $LSG_REFERENCE_DIR, else the
    Makefile's REF default (the recipe that compiles them names the path)."""
    env = os.environ.get("LSG_REFERENCE_DIR")
    if env:
        return env
    with open(os.path.join(HERE, "Makefile")) as f:
        for line in f:
            if line.startswith("REF ?="):
                return line.split("?=", 1)[1].strip()
    return ""


def build(with_ref: bool | None = None) -> None:
    """Compile the oracle (and, where the reference checkout exists, the reference)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    ref_dir = reference_dir()
    if with_ref is None:
        with_ref = os.path.isdir(ref_dir)
    if with_ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_dir}"], check=True)


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(with_ref=False)
        L = C.CDLL(ORACLE_SO)
        L.lsgo_lap_coefficient.argtypes = [_dp, C.c_int]
        L.lsgo_op_init.argtypes = [C.POINTER(OpStruct), C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_double, C.c_double]
        L.lsgo_diag.argtypes = [C.POINTER(OpStruct)]
        L.lsgo_diag.restype = C.c_double
        L.lsgo_apply.argtypes = [C.POINTER(OpStruct), _dp, _dp]
        L.lsgo_pinv_solve.argtypes = [_dp, _dp, _dp, C.c_int]
        L.lsgo_pinv_solve.restype = C.c_int
        L.lsgo_aar.argtypes = [C.POINTER(OpStruct), C.c_int, _dp, _dp, C.c_double, C.c_double,
                               C.c_int, C.c_int, C.c_int, C.c_double, C.POINTER(ResultStruct)]
        for name in ("lsgo_pgr", "lsgo_pl2r"):
            getattr(L, name).argtypes = [C.POINTER(OpStruct), C.c_int, _dp, _dp, C.c_double,
                                         C.c_int, C.c_int, C.c_int, C.c_double,
                                         C.POINTER(ResultStruct)]
        L.lsgo_cg.argtypes = [C.POINTER(OpStruct), C.c_int, _dp, _dp, C.c_int, C.c_double,
                              C.POINTER(ResultStruct)]
        L.lsgo_reference_rhs.argtypes = [C.c_int, C.c_int, C.c_int, _dp]
        _cp = np.ctypeslib.ndpointer(dtype=np.complex128, flags="C_CONTIGUOUS")
        L.lsgo_apply_c.argtypes = [C.POINTER(OpStruct), C.c_double, _cp, _cp]
        L.lsgo_aar_c.argtypes = [C.POINTER(OpStruct), C.c_double, C.c_int, _cp, _cp, C.c_double,
                                 C.c_double, C.c_int, C.c_int, C.c_int, C.c_double,
                                 C.POINTER(ResultStruct)]
        L.lsgo_set_threads.argtypes = [C.c_int]
        L.lsgo_max_threads.restype = C.c_int
        L.lsgo_set_threads(1)
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SO)
        L.refh_rhs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp]
        L.refh_coefficients.argtypes = [C.c_int, _dp]
        L.refh_apply.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp]
        L.refh_solve.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                 _dp, _dp, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                                 C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
        L.refh_solve.restype = C.c_int
        L.refh_pinv.argtypes = [_dp, _dp, _dp, C.c_int]
        _ref = L
    return _ref


# ----------------------------------------------------------------------------- oracle wrappers

def make_op(n, radius=6, a=A_REF, sigma=0.0) -> OpStruct:
    nx, ny, nz = (n, n, n) if np.isscalar(n) else tuple(n)
    op = OpStruct()
    lib().lsgo_op_init(C.byref(op), nx, ny, nz, radius, a, sigma)
    return op


def coefficients(radius: int) -> np.ndarray:
    c = np.zeros(radius + 1)
    lib().lsgo_lap_coefficient(c, radius)
    return c


def apply(x: np.ndarray, radius=6, a=A_REF, sigma=0.0) -> np.ndarray:
    """y = (a*Lap + sigma) x; x shaped (nz, ny, nx) or flat with n given by shape."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    nz, ny, nx = x.shape
    op = make_op((nx, ny, nz), radius, a, sigma)
    y = np.empty_like(x)
    lib().lsgo_apply(C.byref(op), x.reshape(-1), y.reshape(-1))
    return y


def apply_c(x: np.ndarray, radius=6, a=A_REF, sigma=0.0):
    """y = (a*Lap + sigma) x for complex x and complex sigma."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    nz, ny, nx = x.shape
    sg = complex(sigma)
    op = make_op((nx, ny, nz), radius, a, sg.real)
    y = np.empty_like(x)
    lib().lsgo_apply_c(C.byref(op), sg.imag, x.reshape(-1), y.reshape(-1))
    return y


def solve_c(b: np.ndarray, x0=None, *, radius=6, a=A_REF, sigma=0.0, precond=True, omega=0.6,
            beta=0.6, m=7, p=6, max_iter=100000, tol=1e-8):
    """Complex AAR (PETSC_COMPLEX/AAR_Complex.c restated); b shaped (nz, ny, nx)."""
    b = np.ascontiguousarray(b, dtype=np.complex128)
    nz, ny, nx = b.shape
    sg = complex(sigma)
    op = make_op((nx, ny, nz), radius, a, sg.real)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.complex128, copy=True)
    res = ResultStruct()
    lib().lsgo_aar_c(C.byref(op), sg.imag, int(precond), x.reshape(-1), b.reshape(-1), omega, beta,
                     m, p, max_iter, tol, C.byref(res))
    return x, dict(iters=res.iters, relres=res.relres, rhs_norm=res.rhs_norm,
                   converged=bool(res.converged), status=res.status, seconds=res.seconds)


def pinv_solve(A: np.ndarray, b: np.ndarray):
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    st = lib().lsgo_pinv_solve(A.reshape(-1), b, x, b.shape[0])
    return x, st


def reference_rhs(nx, ny=None, nz=None) -> np.ndarray:
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    b = np.empty(nx * ny * nz)
    lib().lsgo_reference_rhs(nx, ny, nz, b)
    return b.reshape(nz, ny, nx)


def solve(solver: str, b: np.ndarray, x0=None, *, radius=6, a=A_REF, sigma=0.0, precond=True,
          omega=0.6, beta=0.6, m=7, p=6, max_iter=100000, tol=1e-8, threads=1):
    """Run one oracle solver; returns (x, result dict).  b shaped (nz, ny, nx)."""
    b = np.ascontiguousarray(b, dtype=np.float64)
    nz, ny, nx = b.shape
    op = make_op((nx, ny, nz), radius, a, sigma)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    res = ResultStruct()
    L = lib()
    L.lsgo_set_threads(threads)
    try:
        xf, bf = x.reshape(-1), b.reshape(-1)
        if solver == "aar":
            L.lsgo_aar(C.byref(op), int(precond), xf, bf, omega, beta, m, p, max_iter, tol, C.byref(res))
        elif solver == "pgr":
            L.lsgo_pgr(C.byref(op), int(precond), xf, bf, omega, m, p, max_iter, tol, C.byref(res))
        elif solver == "pl2r":
            L.lsgo_pl2r(C.byref(op), int(precond), xf, bf, omega, m, p, max_iter, tol, C.byref(res))
        elif solver == "cg":
            L.lsgo_cg(C.byref(op), int(precond), xf, bf, max_iter, tol, C.byref(res))
        else:
            raise ValueError(solver)
    finally:
        L.lsgo_set_threads(1)
    return x, dict(iters=res.iters, relres=res.relres, rhs_norm=res.rhs_norm,
                   converged=bool(res.converged), status=res.status, seconds=res.seconds)


def ref_pinv(A: np.ndarray, b: np.ndarray) -> np.ndarray:
    """The reference's PseudoInverseTimesVec (needs ``make ref``)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    ref().refh_pinv(A.reshape(-1), b, x, b.shape[0])
    return x


def ref_solve(solver: str, b: np.ndarray, x0=None, *, radius=6, a=A_REF, precond=True, omega=0.6,
              beta=0.6, m=7, p=6, max_iter=100000, tol=1e-8):
    """Run the compiled reference solver (needs ``make ref``); same conventions as solve()."""
    b = np.array(b, dtype=np.float64, copy=True)
    nz, ny, nx = b.shape
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    it, rr, sec = C.c_int(0), C.c_double(0), C.c_double(0)
    rc = ref().refh_solve(SOLVERS[solver], nx, ny, nz, radius, a, int(precond), x.reshape(-1),
                          b.reshape(-1), omega, beta, m, p, max_iter, tol, C.byref(it),
                          C.byref(rr), C.byref(sec))
    if rc != 0:
        raise RuntimeError(f"reference {solver} printed no report (rc={rc})")
    return x, dict(iters=it.value, relres=rr.value, seconds=sec.value)


# ----------------------------------------------------------------------------- FFT diagonal solve

def symbol(shape, radius=6, a=A_REF, sigma=0.0, coeff=None):
    """Eigenvalues of the periodic operator a*Lap + sigma on an (nz, ny, nx) grid.

    The operator is a constant-coefficient circulant, so its DFT symbol is
    a*(3 c_0 + sum_p 2 c_p (cos(2 pi p kx/nx) + cos(.. ky ..) + cos(.. kz ..))) + sigma.
    """
    nz, ny, nx = shape
    c = coefficients(radius) if coeff is None else np.asarray(coeff)

    def axis(n):
        k = np.arange(n)
        s = np.zeros(n)
        for p in range(1, radius + 1):
            s += 2.0 * c[p] * np.cos(2.0 * np.pi * p * k / n)
        return s

    lam = (3.0 * c[0] + axis(nz)[:, None, None] + axis(ny)[None, :, None] + axis(nx)[None, None, :])
    return a * lam + sigma


def fft_solve(b: np.ndarray, radius=6, a=A_REF, sigma=0.0, zero_mean=True):
    """Exact solve of (a*Lap + sigma) x = b on the periodic grid (complex sigma allowed).

    For the singular Poisson operator (sigma = 0) the zero mode is set to 0,
    i.e. the mean-free solution is returned.
    """
    lam = symbol(b.shape, radius, a, 0.0) + sigma
    bh = np.fft.fftn(b)
    with np.errstate(divide="ignore", invalid="ignore"):
        xh = bh / lam
    if zero_mean or sigma == 0:
        xh[0, 0, 0] = 0.0 if sigma == 0 else xh[0, 0, 0]
    x = np.fft.ifftn(xh)
    if np.isrealobj(b) and np.isrealobj(np.asarray(sigma)):
        return x.real
    return x


# ----------------------------------------------------------------------------- GMRES(m)

def gmres(b: np.ndarray, x0=None, *, restart=30, tol=1e-8, max_iter=2000, radius=6, a=A_REF,
          sigma=0.0, precond=True):
    """Restarted GMRES(restart), left Jacobi preconditioning, classical
    Gram-Schmidt: the steps of liblsg's lsg_gmres in numpy (test
    infrastructure).  The reference's comparator is PETSc's KSPGMRES
    (PETSC_REAL/main.c:84-122), which is not available here; this restates
    Saad & Schultz's algorithm with the same stopping rules.  Returns (x, dict)."""
    b = np.asarray(b, dtype=np.float64)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    c = coefficients(radius)
    diag = a * 3.0 * c[0] + sigma
    cf = 1.0 / diag if precond else 1.0
    A = lambda v: apply(v, radius, a, sigma)
    bnorm = np.linalg.norm(b)
    tol_abs = tol * bnorm
    m = restart
    iters = 0
    while True:
        r = b - A(x)
        nr = np.linalg.norm(r)
        if not nr > tol_abs or iters >= max_iter:
            return x, dict(iters=iters, relres=nr / bnorm if bnorm > 0 else nr,
                           converged=bool(not nr > tol_abs))
        W = [r]
        s = [np.sign(cf) / nr if cf != 0 else 0.0]
        g = np.zeros(m + 1)
        g[0] = abs(cf) * nr
        H = np.zeros((m + 1, m))
        cs, sn = np.zeros(m), np.zeros(m)
        k = 0
        for j in range(m):
            z = cf * A(s[j] * W[j])
            h = np.array([s[i] * np.dot(W[i].ravel(), z.ravel()) for i in range(j + 1)])
            H[:j + 1, j] = h
            z = z - sum((h[i] * s[i]) * W[i] for i in range(j + 1))
            eta = np.linalg.norm(z)
            H[j + 1, j] = eta
            W.append(z)
            s.append(1.0 / eta if eta > 0 else 0.0)
            for i in range(j):
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                H[i, j] = t
            rr = np.hypot(H[j, j], eta)
            cs[j], sn[j] = (H[j, j] / rr, eta / rr) if rr > 0 else (1.0, 0.0)
            H[j, j] = rr
            H[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            k = j + 1
            iters += 1
            if abs(g[j + 1]) <= tol_abs * abs(cf) or iters >= max_iter or not eta > 0:
                break
        y = np.zeros(k)
        for i in range(k - 1, -1, -1):
            y[i] = (g[i] - H[i, i + 1:k] @ y[i + 1:k]) / H[i, i] if H[i, i] != 0 else 0.0
        x = x + sum((y[i] * s[i]) * W[i] for i in range(k))


def lgmres(b: np.ndarray, x0=None, *, restart=30, aug=2, tol=1e-8, max_iter=2000, radius=6, a=A_REF,
           sigma=0.0, precond=True):
    """LGMRES(m, k) of Baker, Jessup & Manteuffel (SIAM J. Matrix Anal. Appl.
    26, 2005) with the parameters of PETSc's KSPLGMRES defaults, which the
    reference runs on its complex operator (PETSC_COMPLEX/main.c:123-147):
    restart = m = the whole approximation space, m - k Krylov vectors plus the
    error approximations z = x_i - x_{i-1} of the last k cycles (fewer in the
    first cycles), newest first.  Each cycle runs the Arnoldi process on the
    augmented set [v_1 .. v_{m-k}, z_1 .. z_na] (classical Gram-Schmidt,
    Givens rotations, left Jacobi), x += W y, and keeps W y as the newest z.
    Real or complex (Hermitian inner products, complex Givens rotations as in
    gmres_c).  PETSc is absent here; this restates the published algorithm
    with the steps of liblsg's lsg_lgmres.  Returns (x, dict)."""
    cx = np.iscomplexobj(b) or isinstance(sigma, complex)
    dt = np.complex128 if cx else np.float64
    b = np.asarray(b, dtype=dt)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=dt, copy=True)
    c = coefficients(radius)
    if cx:
        sg = complex(sigma)
        cf = 1.0 / (a * 3.0 * c[0] + sg) if precond else 1.0 + 0j
        A = lambda v: apply_c(v, radius, a, sg)
    else:
        cf = 1.0 / (a * 3.0 * c[0] + sigma) if precond else 1.0
        A = lambda v: apply(v, radius, a, sigma)
    acf = abs(cf)
    bnorm = np.linalg.norm(b)
    tol_abs = tol * bnorm
    m, mk = restart, restart - aug
    iters = 0
    Z = []  # (vector, scale), newest first
    while True:
        r = b - A(x)
        nr = np.linalg.norm(r)
        if not nr > tol_abs or iters >= max_iter:
            return x, dict(iters=iters, relres=nr / bnorm if bnorm > 0 else nr,
                           converged=bool(not nr > tol_abs))
        W = [r]
        s = [(1.0 / nr) * (cf / acf)]
        g = np.zeros(m + 1, dtype=dt)
        g[0] = acf * nr
        H = np.zeros((m + 1, m), dtype=dt)
        cs = np.zeros(m)
        sn = np.zeros(m, dtype=dt)
        na = min(len(Z), aug)
        k = 0
        for j in range(mk + na):
            u = s[j] * W[j] if j < mk else Z[j - mk][1] * Z[j - mk][0]
            z = cf * A(u)
            h = np.array([np.conj(s[i]) * np.vdot(W[i].ravel(), z.ravel()) for i in range(j + 1)])
            H[:j + 1, j] = h
            z = z - sum((h[i] * s[i]) * W[i] for i in range(j + 1))
            eta = np.linalg.norm(z)
            W.append(z)
            s.append(1.0 / eta if eta > 0 else 0.0)
            for i in range(j):
                hi, hn = H[i, j], H[i + 1, j]
                H[i, j] = cs[i] * hi + sn[i] * hn
                H[i + 1, j] = cs[i] * hn - np.conj(sn[i]) * hi
            hj = H[j, j]
            if cx:  # c = |h| / rho, s = (h / |h|) eta / rho
                ah = abs(hj)
                rr = np.hypot(ah, eta)
                ph = hj / ah if ah > 0 else 1.0
                cs[j] = ah / rr if rr > 0 else 1.0
                sn[j] = (eta / rr) * ph if rr > 0 else 0.0
                H[j, j] = rr * ph
            else:  # c = h / rho, s = eta / rho
                rr = np.hypot(hj, eta)
                cs[j], sn[j] = (hj / rr, eta / rr) if rr > 0 else (1.0, 0.0)
                H[j, j] = rr
            H[j + 1, j] = 0.0
            g[j + 1] = -np.conj(sn[j]) * g[j]
            g[j] = cs[j] * g[j]
            k = j + 1
            iters += 1
            if abs(g[j + 1]) <= tol_abs * acf or iters >= max_iter or not eta > 0:
                break
        y = np.zeros(k, dtype=dt)
        for i in range(k - 1, -1, -1):
            y[i] = (g[i] - H[i, i + 1:k] @ y[i + 1:k]) / H[i, i] if H[i, i] != 0 else 0.0
        delta = sum((y[i] * s[i]) * W[i] for i in range(min(k, mk)))
        for i in range(mk, k):
            delta = delta + (y[i] * Z[i - mk][1]) * Z[i - mk][0]
        x = x + delta
        nd = np.linalg.norm(delta)
        Z.insert(0, (delta, 1.0 / nd if nd > 0 else 0.0))
        del Z[aug:]


def gmres_c(b: np.ndarray, x0=None, *, restart=30, tol=1e-8, max_iter=2000, radius=6, a=A_REF,
            sigma=0.0, precond=True):
    """Complex restarted GMRES(restart) for the complex-shifted operator
    a*Lap + sigma (sigma complex), left Jacobi (cf = 1 / (3 a c_0 + sigma)),
    classical Gram-Schmidt with Hermitian inner products, complex Givens
    rotations G = [[c, s], [-conj(s), c]] (c = |h| / rho, s = (h / |h|) eta /
    rho): the steps of lsg_gmres on complex vectors.  The reference runs
    PETSc's KSPGMRES on its complex operator (PETSC_COMPLEX/main.c:80-110);
    PETSc is absent, so this restates Saad & Schultz's algorithm."""
    b = np.asarray(b, dtype=np.complex128)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.complex128, copy=True)
    c = coefficients(radius)
    sg = complex(sigma)
    cf = 1.0 / (a * 3.0 * c[0] + sg) if precond else 1.0 + 0j
    A = lambda v: apply_c(v, radius, a, sg)
    bnorm = np.linalg.norm(b)
    tol_abs = tol * bnorm
    m = restart
    iters = 0
    acf = abs(cf)
    while True:
        r = b - A(x)
        nr = np.linalg.norm(r)
        if not nr > tol_abs or iters >= max_iter:
            return x, dict(iters=iters, relres=nr / bnorm if bnorm > 0 else nr,
                           converged=bool(not nr > tol_abs))
        W = [r]
        s = [(1.0 / nr) * (cf / acf)]
        g = np.zeros(m + 1, dtype=np.complex128)
        g[0] = acf * nr
        H = np.zeros((m + 1, m), dtype=np.complex128)
        cs, sn = np.zeros(m), np.zeros(m, dtype=np.complex128)
        k = 0
        for j in range(m):
            z = cf * A(s[j] * W[j])
            h = np.array([np.conj(s[i]) * np.vdot(W[i].ravel(), z.ravel()) for i in range(j + 1)])
            H[:j + 1, j] = h
            z = z - sum((h[i] * s[i]) * W[i] for i in range(j + 1))
            eta = np.linalg.norm(z)
            H[j + 1, j] = eta
            W.append(z)
            s.append(1.0 / eta if eta > 0 else 0.0)
            for i in range(j):
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = cs[i] * H[i + 1, j] - np.conj(sn[i]) * H[i, j]
                H[i, j] = t
            aa = abs(H[j, j])
            rr = np.hypot(aa, eta)
            ph = H[j, j] / aa if aa > 0 else 1.0
            cs[j], sn[j] = (aa / rr, (eta / rr) * ph) if rr > 0 else (1.0, 0.0)
            H[j, j] = rr * ph
            H[j + 1, j] = 0.0
            g[j + 1] = -np.conj(sn[j]) * g[j]
            g[j] = cs[j] * g[j]
            k = j + 1
            iters += 1
            if abs(g[j + 1]) <= tol_abs * acf or iters >= max_iter or not eta > 0:
                break
        y = np.zeros(k, dtype=np.complex128)
        for i in range(k - 1, -1, -1):
            y[i] = (g[i] - H[i, i + 1:k] @ y[i + 1:k]) / H[i, i] if H[i, i] != 0 else 0.0
        x = x + sum((y[i] * s[i]) * W[i] for i in range(k))


def cocg(b: np.ndarray, x0=None, *, tol=1e-8, max_iter=100000, radius=6, a=A_REF, sigma=0.0, precond=True):
    """Conjugate orthogonal CG (van der Vorst & Melissen 1990) for the
    complex-symmetric operator a*Lap + sigma, Jacobi preconditioned: CG with
    the bilinear form u^T v in place of u^H v.  It is BiCG (the reference's
    KSPBICG, PETSC_COMPLEX/main.c:150-175) with the shadow residual conj(r0),
    whose iterates then stay the conjugates of the primal ones, at one
    operator application per step.  Convergence on ||r||_2 / ||b||_2."""
    b = np.asarray(b, dtype=np.complex128)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.complex128, copy=True)
    c = coefficients(radius)
    sg = complex(sigma)
    cf = 1.0 / (a * 3.0 * c[0] + sg) if precond else 1.0 + 0j
    A = lambda v: apply_c(v, radius, a, sg)
    bnorm = np.linalg.norm(b)
    tol_abs = tol * bnorm
    r = b - A(x)
    rho = cf * np.sum(r * r)
    d = np.zeros_like(b)
    beta = 0.0
    it = 0
    nr = np.linalg.norm(r)
    while nr > tol_abs and it < max_iter:
        d = cf * r + beta * d
        q = A(d)
        alpha = rho / np.sum(d * q)
        x = x + alpha * d
        r = r - alpha * q
        it += 1
        rho_new = cf * np.sum(r * r)
        beta = rho_new / rho
        rho = rho_new
        nr = np.linalg.norm(r)
    return x, dict(iters=it, relres=nr / bnorm if bnorm > 0 else nr, converged=bool(not nr > tol_abs))


# ----------------------------------------------------------------------------- AAR on any matrix

def aar_general(matvec, dinv, b, x0=None, *, omega=0.6, beta=0.6, m=7, p=6, tol=1e-8, max_iter=100000,
                precond=None):
    """MPI_REAL/AAR.c:37-177 with any operator `matvec` and Jacobi factors
    `dinv` (1 / diag(A), or ones), in numpy (test infrastructure for the
    general sparse operator path).  `precond(r)`, when given, replaces the
    Jacobi scaling (the PCApply of PETSC_REAL/AAR_Real.c:100-103, e.g. the
    block ICC(0) below).  The m x m solve is the reference's pseudo-inverse
    (`pinv_solve`).  Returns (x, dict(iters, relres))."""
    b = np.asarray(b, dtype=np.float64).ravel()
    n = b.size
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64).ravel()
    tol_abs = tol * np.linalg.norm(b)                 # AAR.c:78-79
    r = b - matvec(x)                                 # AAR.c:80-82
    DX, DF = np.zeros((m, n)), np.zeros((m, n))
    relres = tol_abs + 1.0
    x_old = f_old = None
    it = 1
    while it <= max_iter and relres > tol_abs:        # AAR.c:91
        f = dinv * r if precond is None else precond(r)  # Precondition
        if it > 1:                                    # AAR.c:96-102
            c = (it - 2) % m
            DX[c], DF[c] = x - x_old, f - f_old
        x_old, f_old = x.copy(), f.copy()
        if it % p == 0 and it > 1:                    # AndersonExtrapolation, AAR.c:109-123
            G = DF @ DF.T
            s, _ = pinv_solve(G, DF @ f)
            x = x_old + beta * f - (DX + beta * DF).T @ s
            r = b - matvec(x)
            relres = np.linalg.norm(r)
        else:
            x = x_old + omega * f                     # AAR.c:134-135
            r = b - matvec(x)
        it += 1
    return x, dict(iters=it - 1, relres=relres / np.linalg.norm(b), converged=bool(relres <= tol_abs))


# ---------------------------------------------------------------- block ICC(0)
# PETSC_REAL/AAR_Real.c:58-61 and PETSC_COMPLEX/AAR_Complex.c:63-66 (pc = 1):
# PCICC on each rank's diagonal block of A (MatGetDiagonalBlock), i.e.
# block-Jacobi with incomplete Cholesky, zero fill, on every block.  Here the
# blocks are the (bx, by, bz) boxes tiling the periodic grid (the subdomains a
# Cartesian rank grid would own); couplings that leave a box -- the periodic
# wrap included -- are dropped.  The operator has constant coefficients, so
# every box has the same block matrix and one factor serves all of them.


def icc0_block_factor(block, weights, radius=6, shift=0.0):
    """Incomplete LDL^T of the block matrix (natural order, x fastest; zero fill).

    weights: w[0] (diagonal, 3 a c_0 + sigma) and w[1..radius] (a c_p).  The
    lower neighbours of a point are the star points at distance p = 1..radius
    below it along each axis that lie in the box; two such rows share lower
    neighbours only along their common axis, so
        l(i, i-p e) = (w_p - sum_{q>p} l(i, i-q e) l(i-p e, i-q e) d(i-q e)) / d(i-p e)
        d(i)        = w_0 (1 + shift) - sum_{axis, p} l(i, i-p e)^2 d(i-p e).
    Returns (L, d): L[i, 6 a + p - 1] = l(i, i - p e_a) (0 outside the box), or
    None when a pivot is not positive."""
    bx, by, bz = block
    n = bx * by * bz
    R = radius
    L = np.zeros((n, 3 * 6))
    d = np.zeros(n)
    strides = (1, bx, bx * by)
    for i in range(n):
        c = (i % bx, (i // bx) % by, i // (bx * by))
        acc = weights[0] * (1.0 + shift)
        for a in range(3):
            for p in range(R, 0, -1):          # farthest first: its terms feed the nearer ones
                if c[a] < p:
                    continue
                k = i - p * strides[a]
                t = weights[p]
                for q in range(R, p, -1):
                    if c[a] < q:
                        continue
                    tt = i - q * strides[a]
                    t = t - L[i, 6 * a + q - 1] * L[k, 6 * a + (q - p) - 1] * d[tt]
                L[i, 6 * a + p - 1] = t / d[k]
        for a in range(3):
            for p in range(1, R + 1):
                if c[a] >= p:
                    k = i - p * strides[a]
                    acc = acc - L[i, 6 * a + p - 1] * L[i, 6 * a + p - 1] * d[k]
        if not acc > 0.0:
            return None
        d[i] = acc
    return L, d


def icc0_factor_shifted(block, weights, radius=6):
    """The factor of the first shift in 0, 1e-3, 2e-3, 4e-3, ... (a multiple of
    the diagonal, Manteuffel's remedy for a non-positive pivot) that gives
    positive pivots.  Returns (L, d, shift)."""
    shift = 0.0
    for _ in range(40):
        f = icc0_block_factor(block, weights, radius, shift)
        if f is not None:
            return f[0], f[1], shift
        shift = 1e-3 if shift == 0.0 else 2.0 * shift
    raise RuntimeError("ICC(0): no positive factor")


def icc0_apply(r, shape, block, L, d, radius=6):
    """f = (L D L^T)^-1 r on every box of the (nz, ny, nx) grid: forward
    solve with unit-diagonal L, division by D, backward solve with L^T; sums in
    the fixed order axis x, y, z and p = 1..radius."""
    nz, ny, nx = shape
    bx, by, bz = block
    n = bx * by * bz
    R = radius
    strides = (1, bx, bx * by)
    rb = np.asarray(r, dtype=np.float64).reshape(nz // bz, bz, ny // by, by, nx // bx, bx)
    rb = rb.transpose(0, 2, 4, 1, 3, 5).reshape(-1, n)      # (blocks, points in natural order)
    y = np.zeros_like(rb)
    coords = [(i % bx, (i // bx) % by, i // (bx * by)) for i in range(n)]
    for i in range(n):
        acc = rb[:, i].copy()
        c = coords[i]
        for a in range(3):
            for p in range(1, R + 1):
                if c[a] >= p:
                    acc = acc - L[i, 6 * a + p - 1] * y[:, i - p * strides[a]]
        y[:, i] = acc
    z = y / d
    x = np.zeros_like(rb)
    for i in range(n - 1, -1, -1):
        acc = z[:, i].copy()
        c = coords[i]
        dims = (bx, by, bz)
        for a in range(3):
            for p in range(1, R + 1):
                if c[a] + p < dims[a]:
                    j = i + p * strides[a]
                    acc = acc - L[j, 6 * a + p - 1] * x[:, j]
        x[:, i] = acc
    x = x.reshape(nz // bz, ny // by, nx // bx, bz, by, bx).transpose(0, 3, 1, 4, 2, 5)
    return x.reshape(nz, ny, nx)


def stencil_weights(radius=6, a=A_REF, sigma=0.0):
    c = coefficients(radius)
    return [a * 3.0 * c[0] + sigma] + [a * c[p] for p in range(1, radius + 1)]
