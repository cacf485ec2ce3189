/*
 * lsg.h — native C ABI of liblsg, the GB300 (sm_103a) AAR / PGR / PL2R / CG
 * solvers for the periodic high-order finite-difference operator
 *
 *     A = a * Lap_h + sigma * I,   Lap_h = 3-D periodic central-difference
 *                                  Laplacian of half-width `radius` (FDn)
 *
 * on an nx x ny x nz grid stored x-fastest (flat index i + j*nx + k*nx*ny,
 * the layout of MPI_REAL/system.c:82).  Every vector argument is a DEVICE
 * pointer owned by the caller; the library allocates its own work arrays
 * (cached per device, grid and history size; see lsg_release_workspaces).
 *
 * Plain C: no CUDA or torch types appear here.  `stream` is a cudaStream_t
 * passed as void* (NULL = the legacy default stream).  Every call returns an
 * lsg_status; none of them exits or aborts the process.
 *
 * The drop-in entry points with the reference's own prototypes (AAR, PGR,
 * PL2R, CG on host buffers) are declared in lsg_compat.h.
 */
#ifndef LSG_H
#define LSG_H

#ifdef __cplusplus
extern "C" {
#endif

#define LSG_MAX_RADIUS 8
#define LSG_MAX_M 32

typedef enum lsg_status {
    LSG_OK = 0,
    LSG_NOT_CONVERGED = 1,     /* max_iter reached; the result holds the last residual */
    LSG_NAN_DETECTED = 2,      /* a residual norm or Gram entry became NaN/Inf */
    LSG_BAD_ARG = 3,           /* invalid size / parameter / NULL pointer */
    LSG_CUDA_ERROR = 4,        /* a CUDA call failed (message via lsg_last_error) */
    LSG_TIMEOUT = 5,           /* a bounded device wait gave up */
    LSG_UNSUPPORTED = 6,       /* valid request this build does not serve */
    LSG_NO_MEMORY = 7,         /* device allocation failed */
    LSG_SVD_NO_CONVERGENCE = 8,/* the m x m Jacobi SVD hit its sweep limit */
    LSG_RANGE = 9              /* an FP64 stencil input exceeded the double-float range
                                  (|u| >= 2^127 ||b||); repeat with lsg_set_fp64_arith(1) */
} lsg_status;

typedef enum lsg_dtype {
    LSG_F64 = 0,  /* double vectors, FP64 arithmetic */
    LSG_F32 = 1,  /* float vectors and stencil; reductions and the m x m solve in FP64 */
    LSG_C128 = 2, /* complex double (re, im interleaved) vectors; AAR only */
    LSG_C64 = 3   /* complex float vectors; AAR only */
} lsg_dtype;

/* The operator.  coeff[] are the 1-D Laplacian FD coefficients c_0..c_radius
 * of MPI_REAL/system.c:480-498 (lsg_lap_coefficient fills them). */
typedef struct lsg_operator {
    int n[3];                          /* grid points along x, y, z */
    int radius;                        /* FDn, 1..LSG_MAX_RADIUS */
    double coeff[LSG_MAX_RADIUS + 1];  /* c_0..c_radius */
    double a;                          /* Laplacian scale (the reference passes -1/(4 pi)) */
    double sigma;                      /* diagonal shift, real part; 0 = the reference operator */
    int precond;                       /* 1: Jacobi, f = r / (3 a c_0 + sigma); 0: none */
    double sigma_im;                   /* imaginary part of the shift (complex dtypes only):
                                          A = a Lap + (sigma + i sigma_im) I, the shifted
                                          Helmholtz operator of PETSC_COMPLEX/system.c:209-272 */
} lsg_operator;

/* Solver parameters, named as the reference's arguments (MPI_REAL/AAR.h:18-22). */
typedef struct lsg_params {
    double omega;        /* Richardson relaxation (AAR, PGR, PL2R) */
    double beta;         /* Anderson mixing (AAR) */
    int m;               /* history depth, 1..LSG_MAX_M */
    int p;               /* extrapolation / projection period */
    int max_iter;        /* iteration limit (inner limit for the mixed solver) */
    double tol;          /* stop when ||b - A x|| <= tol * ||b|| */
    /* mixed precision (lsg_aar_mixed) */
    double inner_tol;    /* FP32 residual reduction between FP64 residual replacements (0 = 3e-4) */
    int max_outer;       /* FP64 residual replacements (0 = 50) */
    /* execution */
    int check_every;     /* extrapolation cycles enqueued between convergence reads (0 = auto) */
} lsg_params;

typedef struct lsg_result {
    int iters;           /* iteration count as the reference reports it (AAR.c:153) */
    double relres;       /* last computed ||r|| / ||b|| (the reference's printed value) */
    double rhs_norm;     /* ||b|| */
    int status;          /* lsg_status of the solve */
    int outer_iters;     /* mixed solver: FP64 refinement steps taken */
    int inner_iters;     /* mixed solver: total FP32 iterations */
    double seconds;      /* host wall time of the call */
    long long launches;  /* kernels launched by the call */
    int svd_fallbacks;   /* extrapolations whose m x m solve took the Jacobi SVD
                            (the Gram was not provably well enough conditioned
                            for the LDL^T path) */
} lsg_result;

/* Fills c[0..radius] with the reference FD coefficients.  Returns LSG_BAD_ARG
 * outside 1..LSG_MAX_RADIUS. */
int lsg_lap_coefficient(int radius, double *c);

/* Fills op for the reference operator of half-width `radius` scaled by a,
 * shifted by sigma, with (precond=1) or without Jacobi preconditioning. */
int lsg_operator_init(lsg_operator *op, int nx, int ny, int nz, int radius, double a,
                      double sigma, int precond);

/* Reference parameter defaults: omega = beta = 0.6, m = 7, p = 6, tol = 1e-8,
 * max_iter = 100000 (MPI_REAL/main.c:37, README:18-21). */
void lsg_params_default(lsg_params *prm);

/* Arithmetic of the FP64 stencil passes inside the solvers.  0 (default):
 * double-float -- each double is split into two floats and the 37-point sums
 * run on the FP32 pipe with error-free transformations (result within ~2^-48
 * of sum |w_p| |u|, FP64's own rounding being ~2^-53 of it), because GB300
 * executes FP64 at ~1/64 of its FP32 rate.  Solves asking for tol < 1e-10
 * use FP64 arithmetic regardless (the double-float residual floor is near
 * 1e-13).  1: FP64 arithmetic throughout.  The environment variable
 * LSG_FP64_ARITH=1 sets 1 at load.  Returns the previous mode.  lsg_apply
 * always uses FP64 arithmetic. */
int lsg_set_fp64_arith(int mode);

/* Form of the FP32 (and mixed-precision inner) AAR's Richardson passes, all
 * giving the same residuals, history columns and extrapolation steps bit for
 * bit.  0 (default): the residual ring -- a pass reads r_{k-1} and writes r_k
 * only, into a ring of m + 1 residuals from which the Gram and update kernels
 * rebuild DF_k = (r_k - r_{k-1}) cf and H_k = c r_{k-1} + beta DF_k (m <= 8,
 * p - 1 <= m, grid size a multiple of 4, 16-byte aligned x; otherwise 1).
 * 1: the lean form (r', H, DF stored; x rebuilt at each extrapolation).
 * 2: the x-carrying recurrence (x, r', H, DF stored), whose iterates form 0
 * reproduces bit for bit.  LSG_AAR_FORM sets the value at load.  Returns the
 * previous form, or -1 for a form outside 0..2. */
int lsg_set_aar_form(int form);

/* Stencil march of the FP32 batched Richardson passes: 1 (default) the paired
 * march (two columns per lane, 64-wide tiles) when every grid has an even nx
 * and every x is 8-byte aligned, 0 the one-column march.  Both give the same
 * results bit for bit.  Returns the previous setting. */
int lsg_set_batch_march(int paired);

/* Batched inner products kept on the device: d_out[k] = sum_i conj(x_k[i]) y_k[i]
 * (real dtypes: sum x y; complex: Re, Im at d_out[2k], d_out[2k+1]) for count
 * vectors of n values stored back to back in d_x and d_y, accumulated in FP64
 * (double-float for F32 / C64) in a fixed order, enqueued on `stream` without
 * a host synchronisation.  d_scratch: device doubles, count * lsg_dot_blocks(n)
 * * (2 for complex dtypes, else 1). */
int lsg_dot_blocks(long long n);
int lsg_dot(int dtype, int count, long long n, const void *d_x, const void *d_y, double *d_out,
            double *d_scratch, void *stream);

/* y = A x on the device (replaces MPI_REAL/system.c:80-213). */
int lsg_apply(const lsg_operator *op, int dtype, const void *d_x, void *d_y, void *stream);

/* Solvers.  d_x: initial guess in, solution out.  d_b: right-hand side.
 * dtype selects double or float vectors.  res may be NULL. */
int lsg_aar(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x,
            const void *d_b, lsg_result *res, void *stream);   /* MPI_REAL/AAR.c:37 */
int lsg_pgr(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x,
            const void *d_b, lsg_result *res, void *stream);   /* MPI_REAL/PGR.c:35 */
int lsg_pl2r(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x,
             const void *d_b, lsg_result *res, void *stream);  /* MPI_REAL/PL2R.c:35 */
int lsg_cg(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x,
           const void *d_b, lsg_result *res, void *stream);    /* MPI_REAL/CG.c:33 */

/* AAR (MPI_REAL/AAR.c:37-177) preconditioned with block-Jacobi ICC(0), the
 * reference's pc = 1 (PETSC_REAL/AAR_Real.c:58-61: PCICC on each rank's
 * diagonal block).  The blocks are the block[0] x block[1] x block[2] boxes
 * tiling the grid (the subdomains of a Cartesian rank grid); couplings
 * leaving a box, the periodic wrap included, are dropped.  Each side must
 * divide the grid, a box holds at most 4096 points, radius <= 6.  FP64
 * vectors; op->precond is ignored.  The factor is an incomplete L D L^T with
 * zero fill, natural order, computed once per operator and box shape on the
 * host (a diagonal shift 1e-3 * 2^k is added if a pivot is not positive). */
int lsg_aar_icc(const lsg_operator *op, const lsg_params *prm, const int block[3], double *d_x,
                const double *d_b, lsg_result *res, void *stream);
/* The block ICC(0) factor lsg_aar_icc uses, on host arrays: L[i*18 + 6*axis +
 * p-1] = l(i, i - p e_axis) (0 where that neighbour lies outside the box),
 * d[i] the pivots, i = x + bx (y + by z); *shift the diagonal shift applied
 * (may be NULL).  No GPU needed. */
int lsg_icc_factor(const lsg_operator *op, const int block[3], double *L, double *d, double *shift);

/* General sparse operator: A x = b for a caller's matrix in CSR form on the
 * device (square, n rows, 32-bit offsets and column indices, FP64 values).
 * The reference's AAR accepts any operator through its Lap_Vec_mult callback
 * (MPI_REAL/AAR.c:37, README:25); a GPU solve needs the operator as data.
 * precond = 1: Jacobi with the matrix's diagonal (every a_ii must be
 * non-zero), 0: none.  The row offsets and column indices are checked on the
 * device before use (LSG_BAD_ARG on a malformed matrix). */
typedef struct lsg_csr {
    int n;                  /* rows = columns */
    long long nnz;          /* stored entries, <= 2^31 - 1 */
    const int *row_ptr;     /* n + 1 offsets, row_ptr[0] = 0, row_ptr[n] = nnz */
    const int *col;         /* nnz column indices in 0..n-1 */
    const double *val;      /* nnz values */
    int precond;            /* 1: Jacobi from the diagonal; 0: none */
    int lanes_per_row;      /* 0: chosen from the mean row length; else 1, 4, 8, 16 or 32 */
} lsg_csr;
/* AAR (MPI_REAL/AAR.c:37-177) with the CSR operator; m <= 8. */
int lsg_aar_csr(const lsg_csr *A, const lsg_params *prm, double *d_x, const double *d_b,
                lsg_result *res, void *stream);
/* y = A x for the CSR operator. */
int lsg_apply_csr(const lsg_csr *A, const double *d_x, double *d_y, void *stream);

/* Restarted GMRES(m), prm->m = restart length (the reference's comparator:
 * PETSc KSPGMRES, PETSC_REAL/main.c:84-122 and, on the complex shifted
 * operator, PETSC_COMPLEX/main.c:80-110; PETSc's default restart is 30).
 * Left Jacobi preconditioning, classical Gram-Schmidt (Hermitian inner
 * products and complex Givens rotations for complex vectors); stops when the
 * GMRES residual estimate reaches tol * ||M^-1 b|| and the true residual of
 * the restarted x confirms ||b - A x|| <= tol ||b||.  res->iters counts
 * Arnoldi steps.  Any dtype; omega, beta and p are unused. */
int lsg_gmres(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x,
              const void *d_b, lsg_result *res, void *stream);

/* LGMRES(m, aug) (the reference's KSPLGMRES, PETSC_COMPLEX/main.c:123-147;
 * Baker, Jessup & Manteuffel 2005) with PETSc's convention: prm->m is the
 * whole approximation space of a cycle, m - aug Krylov vectors plus the error
 * approximations x_i - x_{i-1} of the last aug cycles (fewer in the first
 * cycles; PETSc's defaults are m = 30, aug = 2).  Otherwise as lsg_gmres:
 * left Jacobi, classical Gram-Schmidt, any dtype, res->iters counts operator
 * applications.  1 <= aug <= min(4, m - 1). */
int lsg_lgmres(const lsg_operator *op, const lsg_params *prm, int aug, int dtype, void *d_x,
               const void *d_b, lsg_result *res, void *stream);

/* BiCG on the complex-symmetric shifted operator (the reference's KSPBICG,
 * PETSC_COMPLEX/main.c:150-175), in its conjugate orthogonal CG form: with
 * the shadow residual conj(r0) BiCG's shadow iterates are the conjugates of
 * the primal ones, so one operator application per step suffices (van der
 * Vorst & Melissen 1990).  Jacobi preconditioned; stops when ||b - A x|| <=
 * tol ||b|| (checked every step).  dtype LSG_C128 or LSG_C64; m, omega, beta,
 * p unused. */
int lsg_cocg(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x,
             const void *d_b, lsg_result *res, void *stream);

/* Mixed precision: FP64 x and b (lsg_aar_mixed_c: complex128 x and b with a
 * complex64 inner iteration).  One FP32 AAR (FP32 vectors, history and
 * stencil; FP64-class reductions and m x m solve) runs on the correction;
 * each time its residual has dropped by inner_tol (or reached tol) the
 * correction is folded into x (FP64), r = b - A x is recomputed in FP64 and
 * the FP32 iteration resumes from it with its history intact.  With a
 * non-zero shift sigma the constant mode is set exactly before each
 * replacement (mean(x) = mean(b) / sigma: the periodic operator maps the
 * constant vector to sigma times itself).  Stops when the FP64 residual
 * satisfies tol.  res->iters counts FP32 iterations, res->outer_iters the
 * FP64 residual replacements. */
int lsg_aar_mixed(const lsg_operator *op, const lsg_params *prm, double *d_x, const double *d_b,
                  lsg_result *res, void *stream);
int lsg_aar_mixed_c(const lsg_operator *op, const lsg_params *prm, void *d_x, const void *d_b,
                    lsg_result *res, void *stream);

/* Batched AAR: `count` independent solves, each with its own operator (grid
 * size, shift, coefficients) and its own x / b (device pointers), sharing
 * prm (omega, beta, m <= 8, p, tol, max_iter).  Every kernel launch covers
 * all unfinished instances and one extrapolation cycle (p iterations) is
 * replayed as a CUDA graph; each instance follows the single solve's
 * iteration (MPI_REAL/AAR.c:37-177), its result in res[i] (res may be NULL).
 * The reference has no batched entry point: its caller loops over AAR().
 * lsg_aar_mixed_batched: dtype LSG_F64 (FP32 inner iteration) or LSG_C128
 * (complex64 inner), the refinement of lsg_aar_mixed per instance.
 * Returns LSG_OK when every instance converged, else the first failure. */
int lsg_aar_batched(const lsg_operator *ops, int count, const lsg_params *prm, int dtype,
                    void *const *d_x, const void *const *d_b, lsg_result *res, void *stream);
int lsg_aar_mixed_batched(const lsg_operator *ops, int count, const lsg_params *prm, int dtype,
                          void *const *d_x, const void *const *d_b, lsg_result *res, void *stream);

/* Autotuner of the Richardson stencil pass (no counterpart in the reference,
 * whose operator is a fixed host loop, MPI_REAL/system.c:189-204).  Times
 * every candidate launch shape -- xy tile variant (threads_y x
 * rows_per_thread rows of 32 columns) and z planes per block -- for the grid
 * of `op` and vector type `dtype` on the device, caches the fastest, and
 * reports it.  Solves on that grid then use the cached shape.  Radius 6. */
typedef struct lsg_tune_info {
    int tile;             /* tile variant index; 3, 4: the FP32 two-columns-per-lane
                             march (tile = 64 x (threads_y * rows_per_thread)) */
    int threads_y;        /* block = 32 x threads_y threads */
    int rows_per_thread;  /* tile = 32 x (threads_y * rows_per_thread) columns */
    int lz;               /* z planes per block */
    double us_best;       /* measured time per launch of the chosen shape */
    double us_default;    /* measured time of the default shape */
    int candidates;       /* shapes timed */
} lsg_tune_info;
int lsg_autotune(const lsg_operator *op, int dtype, lsg_tune_info *info, void *stream);
/* 0: default shapes; 1: use cached shapes (the default); 2: also tune every
 * (dtype, grid) a solve meets for the first time.  LSG_AUTOTUNE=<mode> in the
 * environment sets the initial mode. */
int lsg_set_autotune(int mode);
/* Text cache of tuned shapes; load adds the file's entries (count: entries read, may be NULL). */
int lsg_autotune_save(const char *path);
int lsg_autotune_load(const char *path, int *count);

/* Bounds-checked build (built with LSG_BOUNDS=1): *first_bad = the first
 * out-of-range global or shared index a stencil march met since the library
 * loaded, or -1 when none (the access was skipped, nothing faulted).  The
 * normal build returns LSG_UNSUPPORTED and sets -1.  first_bad may be NULL. */
int lsg_bounds_errors(long long *first_bad);

/* m x m pseudo-inverse solve with the reference's semantics
 * (x = V diag(1/w) V^T b, w < m*wmax*2.22044605e-16 dropped; MPI_REAL/tools.c:52-105),
 * computed on the device by one warp.  A row-major, device pointers. */
int lsg_pinv_solve(const double *d_A, const double *d_b, double *d_x, int m, void *stream);

/* The same solve without any device allocation (no counterpart in the
 * reference, whose solver mallocs its work arrays on every call).  For
 * callers that must not call cudaMalloc -- device memory already owned by an
 * external pool or capped per client, or a loop that cannot pay for an
 * allocation per call -- the kernel's status word lives in a 256-byte static
 * device array that every GPU loading the library holds until exit.  m above
 * LSG_MAX_M is rejected with LSG_BAD_ARG.  The first call on a device looks up
 * that array's address; the address is cached for the life of the process,
 * so the call must not be used after cudaDeviceReset on that device.  Calls share the array: calls that overlap
 * on the GPU race.  Each call waits for `stream` (it reads the status word
 * back before returning). */
int lsg_pinv_solve_noalloc(const double *d_A, const double *d_b, double *d_x, int m,
                           void *stream);

/* Per-kernel-class device time, measured with CUDA events recorded on the
 * solve's stream around each launch while profiling is on. */
enum lsg_kernel_class {
    LSG_K_RICHARDSON = 0, /* fused Richardson stencil step */
    LSG_K_RESIDUAL = 1,   /* residual / operator stencil */
    LSG_K_GRAM = 2,       /* history Gram reduction */
    LSG_K_UPDATE = 3,     /* extrapolation / projection / CG vector updates */
    LSG_K_SMALL = 4,      /* single-block finalize and m x m solve */
    LSG_K_CG = 5,         /* CG direction + operator stencil */
    LSG_K_REFINE = 6,     /* FP64 refinement residual and correction */
    LSG_K_PRECOND = 7,    /* block ICC(0) preconditioner application */
    LSG_K_CLASSES = 8
};
typedef struct lsg_kernel_stats {
    long long launches[LSG_K_CLASSES];
    double ms[LSG_K_CLASSES];
} lsg_kernel_stats;
/* on = 1 starts collecting (and clears the totals), 0 stops. */
int lsg_profile(int on);
/* Copies the totals collected so far. */
int lsg_profile_read(lsg_kernel_stats *stats);

/* Frees every cached work array on the current device. */
int lsg_release_workspaces(void);

/* Status of the last compat-entry-point call on this thread (AAR/PGR/PL2R/CG
 * return void) and a human-readable message for the last failure. */
int lsg_last_status(void);
const char *lsg_last_error(void);
const char *lsg_status_string(int status);

/* Library version string. */
const char *lsg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LSG_H */
