/*
 * lsg_oracle.c — CPU oracle for the periodic-stencil AAR / PGR / PL2R / CG
 * solvers.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py may load this library, and only as the checker or
 * as the timed CPU baseline.  The product library (liblsg.so) never links,
 * loads or calls it.
 *
 * It restates, in plain C99, the single-rank algorithms of
 * YaphetS-jx/Linear-Solver MPI_REAL:
 *   - FD coefficients           MPI_REAL/system.c:480-498   lsgo_lap_coefficient
 *   - periodic a*Lap*x           MPI_REAL/system.c:189-204   lsgo_apply
 *   - Jacobi preconditioner      MPI_REAL/system.c:222-227   (diag passed as in AAR.c:94)
 *   - 2-norm / dot               MPI_REAL/tools.c:18-43
 *   - pinv(A)*b                  MPI_REAL/tools.c:52-105, 325-335   lsgo_pinv_solve
 *   - AAR + Anderson step        MPI_REAL/AAR.c:37-177, 185-232     lsgo_aar
 *   - PGR + Galerkin step        MPI_REAL/PGR.c:35-173, 181-218     lsgo_pgr
 *   - PL2R + L2 step             MPI_REAL/PL2R.c:35-172, 180-218    lsgo_pl2r
 *   - Jacobi PCG                 MPI_REAL/CG.c:33-175               lsgo_cg
 *   - reference RHS              MPI_REAL/system.c:452-468          lsgo_reference_rhs
 *   - complex AAR              PETSC_COMPLEX/AAR_Complex.c:31-199, 207-246  lsgo_aar_c
 * plus a diagonal shift sigma (A = a*Lap + sigma*I, complex for lsgo_aar_c)
 * used by the shifted configurations; sigma = 0 is the reference operator.
 * The complex path's reference needs PETSc and MKL (not buildable here); its
 * restatement is checked against the exact FFT solve and against the real
 * AAR, which it must reproduce for real sigma and b.
 *
 * Arithmetic is written in the reference's evaluation order and the file is
 * compiled with -ffp-contract=off, so the stencil, the vector updates and
 * the serial reductions round exactly as the reference does on a machine
 * without fused multiply-add.  The m x m pseudo-inverse is computed by a
 * one-sided Jacobi SVD written here from the mathematics (Hestenes 1958);
 * it reproduces the reference's pinv semantics (x = V diag(1/w) V^T b with
 * singular values below m * wmax * 2.22044605e-16 dropped, tools.c:325-335)
 * up to rounding, not its Golub-Reinsch code.
 *
 * OpenMP (when compiled with -fopenmp) parallelises the stencil and the
 * point-wise loops for the timed CPU baseline; lsgo_set_threads(1) gives the
 * serial, reference-order reductions the parity tests use.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define LSGO_MAXR 16
#define LSGO_MAXM 64

typedef struct {
    int n[3];                     /* grid points per axis, x fastest */
    int radius;                   /* FDn */
    double coeff[LSGO_MAXR + 1];  /* 1-D Laplacian FD coefficients c_0..c_R */
    double a;                     /* operator scale */
    double sigma;                 /* real diagonal shift */
} lsgo_op;

typedef struct {
    int iters;        /* iteration count as the reference reports it */
    double relres;    /* last computed ||r|| / ||b|| */
    double rhs_norm;  /* ||b|| */
    int converged;    /* relres <= tol */
    int status;       /* 0 ok, 1 not converged, 2 svd did not converge */
    double seconds;   /* wall time of the iteration loop */
} lsgo_result;

static int g_threads = 1;

void lsgo_set_threads(int t)
{
    g_threads = t < 1 ? 1 : t;
#ifdef _OPENMP
    omp_set_num_threads(g_threads);
#endif
}

int lsgo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* system.c:480-498: c_0 = -sum 2/p^2, c_p = 2 (-1)^(p+1) (FDn!/(FDn-p)!) / ((FDn+p)!/FDn!) / p^2,
 * evaluated with the same products so the coefficients agree bit for bit. */
void lsgo_lap_coefficient(double *c, int fdn)
{
    int i, p;
    c[0] = 0.0;
    for (p = 1; p <= fdn; p++) c[0] += -(2.0 / (p * p));
    for (p = 1; p <= fdn; p++) {
        double nr = 1, dr = 1;
        for (i = fdn - p + 1; i <= fdn; i++) nr *= i;
        for (i = fdn + 1; i <= fdn + p; i++) dr *= i;
        c[p] = 2 * pow(-1, p + 1) * (nr / dr) / (p * p);
    }
}

void lsgo_op_init(lsgo_op *op, int nx, int ny, int nz, int radius, double a, double sigma)
{
    memset(op, 0, sizeof(*op));
    op->n[0] = nx; op->n[1] = ny; op->n[2] = nz;
    op->radius = radius;
    op->a = a;
    op->sigma = sigma;
    lsgo_lap_coefficient(op->coeff, radius);
}

/* Jacobi diagonal: the reference passes a*(3*coeff_lap[0]) (AAR.c:94). */
double lsgo_diag(const lsgo_op *op) { return op->a * (3 * op->coeff[0]) + op->sigma; }

/* y = (a*Lap + sigma) x on the periodic grid, neighbour order and rounding
 * of system.c:195-202 (center term first, then per distance the six
 * neighbours -x,+x,-y,+y,-z,+z summed left to right and scaled). */
void lsgo_apply(const lsgo_op *op, const double *x, double *y)
{
    const int nx = op->n[0], ny = op->n[1], nz = op->n[2], R = op->radius;
    double w[LSGO_MAXR + 1];
    long k;
    for (int p = 0; p <= R; p++) w[p] = op->a * op->coeff[p];
#pragma omp parallel for schedule(static)
    for (k = 0; k < nz; k++) {
        for (int j = 0; j < ny; j++) {
            for (int i = 0; i < nx; i++) {
                const long c = i + (long)nx * (j + (long)ny * k);
                double v = x[c] * 3 * w[0];
                for (int p = 1; p <= R; p++) {
                    const int im = (i - p + p * nx) % nx, ip = (i + p) % nx;
                    const int jm = (j - p + p * ny) % ny, jp = (j + p) % ny;
                    const int km = (int)((k - p + (long)p * nz) % nz), kp = (int)((k + p) % nz);
                    v += (x[im + (long)nx * (j + (long)ny * k)] + x[ip + (long)nx * (j + (long)ny * k)]
                          + x[i + (long)nx * (jm + (long)ny * k)] + x[i + (long)nx * (jp + (long)ny * k)]
                          + x[i + (long)nx * (j + (long)ny * km)] + x[i + (long)nx * (j + (long)ny * kp)]) * w[p];
                }
                if (op->sigma != 0.0) v += op->sigma * x[c];
                y[c] = v;
            }
        }
    }
}

/* tools.c:18-28 / 35-43: serial sums in index order when run on one thread. */
static double dot(const double *a, const double *b, long n)
{
    double s = 0;
    long k;
    if (g_threads == 1) {
        for (k = 0; k < n; k++) s = s + a[k] * b[k];
        return s;
    }
#pragma omp parallel for schedule(static) reduction(+ : s)
    for (k = 0; k < n; k++) s += a[k] * b[k];
    return s;
}

static double norm2(const double *a, long n) { return sqrt(dot(a, a, n)); }

static void precondition(double diag, double *r, long n)
{
    long k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < n; k++) r[k] /= diag;
}

/*
 * x = pinv-as-the-reference-defines-it(A) * b for an m x m matrix A
 * (row-major, A[i*m+j] = A(i,j)).
 *
 * The reference factors A = U W V^T and then, because it assumes a square
 * symmetric matrix, uses V where U belongs (tools.c:325-329):
 *     x = V diag(1/w_j) V^T b,   w_j < m * wmax * 2.22044605e-16  ->  term dropped.
 * For the symmetric positive semi-definite Gram matrices of AAR and PL2R this
 * is the Moore-Penrose pseudo-inverse; for PGR's non-symmetric DX^T DF it is
 * (A^T A)^{+1/2} b, and that is what is reproduced here.
 *
 * One-sided Jacobi: rotate column pairs of a working copy G = A V until all
 * columns are mutually orthogonal; then w_j = ||G(:,j)|| and V holds the
 * right singular vectors.  Returns 0 on success, 2 if the sweep limit hit.
 */
static int pinv_cut(const double *A, const double *b, double *x, int m, double cut);

int lsgo_pinv_solve(const double *A, const double *b, double *x, int m)
{
    return pinv_cut(A, b, x, m, m * 2.22044605e-16);
}

/* As lsgo_pinv_solve with the cutoff w < cut * wmax. */
static int pinv_cut(const double *A, const double *b, double *x, int m, double cut)
{
    double G[LSGO_MAXM * LSGO_MAXM], V[LSGO_MAXM * LSGO_MAXM], w[LSGO_MAXM], t[LSGO_MAXM];
    int i, j, k, sweep, rotated = 1, status = 0;
    const double eps = 2.22044605e-16;
    if (m < 1 || m > LSGO_MAXM) return 3;
    memcpy(G, A, sizeof(double) * m * m);
    for (i = 0; i < m; i++)
        for (j = 0; j < m; j++) V[i * m + j] = (i == j) ? 1.0 : 0.0;

    for (sweep = 0; sweep < 80 && rotated; sweep++) {
        rotated = 0;
        for (i = 0; i < m - 1; i++) {
            for (j = i + 1; j < m; j++) {
                double al = 0, be = 0, ga = 0, zeta, tt, c, s;
                for (k = 0; k < m; k++) {
                    al += G[k * m + i] * G[k * m + i];
                    be += G[k * m + j] * G[k * m + j];
                    ga += G[k * m + i] * G[k * m + j];
                }
                if (ga == 0.0 || fabs(ga) <= eps * sqrt(al * be)) continue;
                rotated = 1;
                zeta = (be - al) / (2.0 * ga);
                if (fabs(zeta) > 1e150) tt = 0.5 / zeta;
                else tt = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                c = 1.0 / sqrt(1.0 + tt * tt);
                s = c * tt;
                for (k = 0; k < m; k++) {
                    double gi = G[k * m + i], gj = G[k * m + j];
                    G[k * m + i] = c * gi - s * gj;
                    G[k * m + j] = s * gi + c * gj;
                    double vi = V[k * m + i], vj = V[k * m + j];
                    V[k * m + i] = c * vi - s * vj;
                    V[k * m + j] = s * vi + c * vj;
                }
            }
        }
    }
    if (rotated) status = 2;

    double wmax = 0;
    for (j = 0; j < m; j++) {
        double s = 0;
        for (k = 0; k < m; k++) s += G[k * m + j] * G[k * m + j];
        w[j] = sqrt(s);
        if (w[j] > wmax) wmax = w[j];
    }
    const double wmin = cut * wmax;
    for (j = 0; j < m; j++) {
        double s = 0;
        if (w[j] >= wmin && w[j] > 0) {
            for (i = 0; i < m; i++) s += V[i * m + j] * b[i];
            s /= w[j];
        }
        t[j] = s;
    }
    for (i = 0; i < m; i++) {
        double s = 0;
        for (j = 0; j < m; j++) s += V[i * m + j] * t[j];
        x[i] = s;
    }
    return status;
}

/* Zeroed work array, first touched by the OpenMP threads that will use it
 * (so its pages are mapped -- and placed near those threads -- before a
 * solver's timer starts: a bounded sample of iterations then measures the
 * steady state, not the page faults of the first writes). */
static void *xcalloc(long n, size_t sz)
{
    const size_t bytes = (size_t)(n > 0 ? n : 1) * sz;
    char *p = malloc(bytes);
    long i;
    const long chunks = (long)((bytes + 65535) / 65536);
    if (!p) abort();
#pragma omp parallel for schedule(static)
    for (i = 0; i < chunks; i++) {
        const size_t off = (size_t)i * 65536;
        memset(p + off, 0, bytes - off < 65536 ? bytes - off : 65536);
    }
    return p;
}

/* AAR.c:37-177 with AndersonExtrapolation AAR.c:185-232. */
int lsgo_aar(const lsgo_op *op, int precond, double *x, const double *rhs, double omega,
             double beta, int m, int p, int max_iter, double tol, lsgo_result *res)
{
    const long np = (long)op->n[0] * op->n[1] * op->n[2];
    const double diag = lsgo_diag(op);
    double *f = xcalloc(np, 8), *x_old = xcalloc(np, 8), *f_old = xcalloc(np, 8);
    double *am = xcalloc(np, 8);
    double *DX = xcalloc(np * m, 8), *DF = xcalloc(np * m, 8);
    double FtF[LSGO_MAXM * LSGO_MAXM], Ftf[LSGO_MAXM], svec[LSGO_MAXM];
    double relres = tol + 1, rhs_norm, t0;
    int iter = 1, col, status = 0;
    long i;

    if (m > LSGO_MAXM) m = LSGO_MAXM;
    rhs_norm = norm2(rhs, np);
    tol *= rhs_norm;
    lsgo_apply(op, x, f);
#pragma omp parallel for schedule(static)
    for (i = 0; i < np; i++) f[i] = rhs[i] - f[i];

    t0 = now_s();
    while (relres > tol && iter <= max_iter) {
        if (precond) precondition(diag, f, np);
        if (iter > 1) {
            col = (iter - 2) % m;
#pragma omp parallel for schedule(static)
            for (i = 0; i < np; i++) {
                DX[col * np + i] = x[i] - x_old[i];
                DF[col * np + i] = f[i] - f_old[i];
            }
        }
        memcpy(x_old, x, sizeof(double) * np);
        memcpy(f_old, f, sizeof(double) * np);

        if (iter % p == 0 && iter > 1) {
            int a, b;
            for (b = 0; b < m; b++)
                for (a = 0; a <= b; a++) {
                    double s = dot(DF + a * np, DF + b * np, np);
                    FtF[b * m + a] = s;
                    FtF[a * m + b] = s;
                }
            for (b = 0; b < m; b++) Ftf[b] = dot(DF + b * np, f, np);
            if (lsgo_pinv_solve(FtF, Ftf, svec, m)) status = 2;
#pragma omp parallel for schedule(static)
            for (i = 0; i < np; i++) {
                double s = 0;
                for (int jj = 0; jj < m; jj++) s = s + (DX[jj * np + i] + beta * DF[jj * np + i]) * svec[jj];
                am[i] = s;
            }
#pragma omp parallel for schedule(static)
            for (i = 0; i < np; i++) x[i] = x_old[i] + beta * f[i] - am[i];
            lsgo_apply(op, x, f);
#pragma omp parallel for schedule(static)
            for (i = 0; i < np; i++) f[i] = rhs[i] - f[i];
            relres = norm2(f, np);
        } else {
#pragma omp parallel for schedule(static)
            for (i = 0; i < np; i++) x[i] = x_old[i] + omega * f[i];
            lsgo_apply(op, x, f);
#pragma omp parallel for schedule(static)
            for (i = 0; i < np; i++) f[i] = rhs[i] - f[i];
        }
        iter = iter + 1;
    }
    if (res) {
        res->seconds = now_s() - t0;
        res->iters = iter - 1;
        res->rhs_norm = rhs_norm;
        res->relres = relres / rhs_norm;
        res->converged = relres <= tol;
        res->status = status ? status : (res->converged ? 0 : 1);
    }
    free(f); free(x_old); free(f_old); free(am); free(DX); free(DF);
    return res ? res->status : 0;
}

/* PGR.c:35-173 (galerkin = 1, Galerkin_Richardson PGR.c:181-218) and
 * PL2R.c:35-172 (galerkin = 0, L2_Richardson PL2R.c:180-218). */
static int periodic_richardson(int galerkin, const lsgo_op *op, int precond, double *x,
                               const double *rhs, double omega, int m, int p, int max_iter,
                               double tol, lsgo_result *res)
{
    const long np = (long)op->n[0] * op->n[1] * op->n[2];
    const double diag = lsgo_diag(op);
    double *Ax = xcalloc(np, 8), *Ax_old = xcalloc(np, 8), *f = xcalloc(np, 8);
    double *x_old = xcalloc(np, 8);
    double *DX = xcalloc(np * m, 8), *DF = xcalloc(np * m, 8);
    double M[LSGO_MAXM * LSGO_MAXM], h[LSGO_MAXM], svec[LSGO_MAXM];
    double relres = tol + 1, rhs_norm, t0;
    int iter = 1, col, status = 0;
    long i;

    if (m > LSGO_MAXM) m = LSGO_MAXM;
    rhs_norm = norm2(rhs, np);
    tol *= rhs_norm;
    lsgo_apply(op, x, Ax);
#pragma omp parallel for schedule(static)
    for (i = 0; i < np; i++) f[i] = rhs[i] - Ax[i];

    t0 = now_s();
    while (relres > tol && iter <= max_iter) {
        if (precond) precondition(diag, f, np);
#pragma omp parallel for schedule(static)
        for (i = 0; i < np; i++) {
            x_old[i] = x[i];
            Ax_old[i] = Ax[i];
            x[i] += (omega * f[i]);
        }
        lsgo_apply(op, x, Ax);
#pragma omp parallel for schedule(static)
        for (i = 0; i < np; i++) f[i] = rhs[i] - Ax[i];

        col = (iter - 2 + m) % m;
#pragma omp parallel for schedule(static)
        for (i = 0; i < np; i++) {
            DX[col * np + i] = x[i] - x_old[i];
            DF[col * np + i] = Ax[i] - Ax_old[i];
        }

        if (iter % p == 0) {
            int a, b;
            if (galerkin) {
                for (b = 0; b < m; b++)
                    for (a = 0; a < m; a++) M[a * m + b] = dot(DX + a * np, DF + b * np, np);
                for (b = 0; b < m; b++) h[b] = dot(DX + b * np, f, np);
            } else {
                for (b = 0; b < m; b++)
                    for (a = 0; a <= b; a++) {
                        double s = dot(DF + a * np, DF + b * np, np);
                        M[b * m + a] = s;
                        M[a * m + b] = s;
                    }
                for (b = 0; b < m; b++) h[b] = dot(DF + b * np, f, np);
            }
            if (lsgo_pinv_solve(M, h, svec, m)) status = 2;
            for (a = 0; a < m; a++) {
                const double sa = svec[a];
#pragma omp parallel for schedule(static)
                for (i = 0; i < np; i++) {
                    x[i] = x[i] + DX[a * np + i] * sa;
                    Ax[i] = Ax[i] + DF[a * np + i] * sa;
                }
            }
#pragma omp parallel for schedule(static)
            for (i = 0; i < np; i++) {
                DX[col * np + i] = x[i] - x_old[i];
                DF[col * np + i] = Ax[i] - Ax_old[i];
            }
        }
#pragma omp parallel for schedule(static)
        for (i = 0; i < np; i++) f[i] = rhs[i] - Ax[i];
        if (iter % p == 0) relres = norm2(f, np);
        iter = iter + 1;
    }
    if (res) {
        res->seconds = now_s() - t0;
        res->iters = iter - 1;
        res->rhs_norm = rhs_norm;
        res->relres = relres / rhs_norm;
        res->converged = relres <= tol;
        res->status = status ? status : (res->converged ? 0 : 1);
    }
    free(Ax); free(Ax_old); free(f); free(x_old); free(DX); free(DF);
    return res ? res->status : 0;
}

int lsgo_pgr(const lsgo_op *op, int precond, double *x, const double *rhs, double omega, int m,
             int p, int max_iter, double tol, lsgo_result *res)
{
    return periodic_richardson(1, op, precond, x, rhs, omega, m, p, max_iter, tol, res);
}

int lsgo_pl2r(const lsgo_op *op, int precond, double *x, const double *rhs, double omega, int m,
              int p, int max_iter, double tol, lsgo_result *res)
{
    return periodic_richardson(0, op, precond, x, rhs, omega, m, p, max_iter, tol, res);
}

/* CG.c:33-175: Jacobi PCG with the true residual recomputed every 50 steps. */
int lsgo_cg(const lsgo_op *op, int precond, double *x, const double *b, int max_iter, double tol,
            lsgo_result *res)
{
    const long np = (long)op->n[0] * op->n[1] * op->n[2];
    const double diag = lsgo_diag(op);
    double *r = xcalloc(np, 8), *d = xcalloc(np, 8), *s = xcalloc(np, 8), *q = xcalloc(np, 8);
    double delta_new, delta_old, alpha, beta, relres, b2, t0;
    int iter_count = 0;
    long i;

    b2 = norm2(b, np);
    lsgo_apply(op, x, r);
#pragma omp parallel for schedule(static)
    for (i = 0; i < np; i++) {
        r[i] = b[i] - r[i];
        d[i] = r[i];
    }
    if (precond) precondition(diag, d, np);
    delta_new = dot(r, d, np);
    relres = precond ? norm2(r, np) : sqrt(delta_new);
    tol *= b2;

    t0 = now_s();
    while (iter_count < max_iter && relres > tol) {
        lsgo_apply(op, d, q);
        alpha = dot(d, q, np);
        alpha = delta_new / alpha;
#pragma omp parallel for schedule(static)
        for (i = 0; i < np; i++) x[i] = x[i] + alpha * d[i];
        if ((iter_count % 50) == 0) {
            lsgo_apply(op, x, r);
#pragma omp parallel for schedule(static)
            for (i = 0; i < np; i++) {
                r[i] = b[i] - r[i];
                s[i] = r[i];
            }
        } else {
#pragma omp parallel for schedule(static)
            for (i = 0; i < np; i++) {
                r[i] = r[i] - alpha * q[i];
                s[i] = r[i];
            }
        }
        if (precond) precondition(diag, s, np);
        delta_old = delta_new;
        delta_new = dot(r, s, np);
        relres = precond ? norm2(r, np) : sqrt(delta_new);
        beta = delta_new / delta_old;
#pragma omp parallel for schedule(static)
        for (i = 0; i < np; i++) d[i] = s[i] + beta * d[i];
        iter_count++;
    }
    if (res) {
        res->seconds = now_s() - t0;
        res->iters = iter_count;
        res->rhs_norm = b2;
        res->relres = relres / b2;
        res->converged = relres <= tol;
        res->status = res->converged ? 0 : 1;
    }
    free(r); free(d); free(s); free(q);
    return res ? res->status : 0;
}

/* system.c:452-468: rhs(g) = 2 rand()/RAND_MAX after srand(g + 1), g the
 * global x-fastest index, then the mean is subtracted.  Uses the C library's
 * own srand/rand, as the reference does. */
void lsgo_reference_rhs(int nx, int ny, int nz, double *rhs)
{
    const long n = (long)nx * ny * nz;
    double sum = 0;
    long g;
    for (g = 0; g < n; g++) {
        srand((unsigned)(g + 1));
        rhs[g] = 2 * (double)(rand()) / (double)(RAND_MAX);
        sum += rhs[g];
    }
    sum /= (double)n;
    for (g = 0; g < n; g++) rhs[g] -= sum;
}

/* ---------------------------------------------------------------- complex */

/* y = (a*Lap + (sigma + i sigma_im)) x, complex vectors. */
void lsgo_apply_c(const lsgo_op *op, double sigma_im, const double complex *x, double complex *y)
{
    const int nx = op->n[0], ny = op->n[1], nz = op->n[2], R = op->radius;
    double w[LSGO_MAXR + 1];
    const double complex shift = op->sigma + I * sigma_im;
    long k;
    for (int p = 0; p <= R; p++) w[p] = op->a * op->coeff[p];
#pragma omp parallel for schedule(static)
    for (k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const long c = i + (long)nx * (j + (long)ny * k);
                double complex v = x[c] * 3 * w[0];
                for (int p = 1; p <= R; p++) {
                    const int im = (i - p + p * nx) % nx, ip = (i + p) % nx;
                    const int jm = (j - p + p * ny) % ny, jp = (j + p) % ny;
                    const int km = (int)((k - p + (long)p * nz) % nz), kp = (int)((k + p) % nz);
                    v += (x[im + (long)nx * (j + (long)ny * k)] + x[ip + (long)nx * (j + (long)ny * k)]
                          + x[i + (long)nx * (jm + (long)ny * k)] + x[i + (long)nx * (jp + (long)ny * k)]
                          + x[i + (long)nx * (j + (long)ny * km)] + x[i + (long)nx * (j + (long)ny * kp)]) * w[p];
                }
                y[c] = v + shift * x[c];
            }
}

static double complex zdot(const double complex *a, const double complex *b, long n) /* a^H b */
{
    double complex s = 0;
    for (long k = 0; k < n; k++) s += conj(a[k]) * b[k];
    return s;
}

/* PETSC_COMPLEX/AAR_Complex.c:31-199 with Anderson (:207-246): Jacobi on the
 * complex diagonal 3 a c_0 + sigma; Gram G(i,j) = DF_i^H DF_j, rhs DF_i^H res;
 * the m x m minimum-norm least-squares solve of LAPACKE_zgelsd with rcond -1
 * (singular values below eps * sigma_max dropped), computed here through the
 * real 2m x 2m representation of the Hermitian G. */
int lsgo_aar_c(const lsgo_op *op, double sigma_im, int precond, double complex *x,
               const double complex *b, double omega, double beta, int m, int p, int max_iter,
               double tol, lsgo_result *res)
{
    const long np = (long)op->n[0] * op->n[1] * op->n[2];
    const double complex diag = op->a * (3 * op->coeff[0]) + op->sigma + I * sigma_im;
    double complex *r = calloc(np, sizeof(double complex)), *x_old = calloc(np, sizeof(double complex));
    double complex *f_old = calloc(np, sizeof(double complex));
    double complex *DX = calloc(np * m, sizeof(double complex)), *DF = calloc(np * m, sizeof(double complex));
    double Gr[4 * LSGO_MAXM * LSGO_MAXM], hr[2 * LSGO_MAXM], sr[2 * LSGO_MAXM];
    double b2 = 0, r2 = tol + 1, t0;
    int iter = 1, status = 0;
    long i;
    if (!r || !x_old || !f_old || !DX || !DF) abort();
    if (m > LSGO_MAXM / 2) m = LSGO_MAXM / 2;
    for (i = 0; i < np; i++) b2 += creal(conj(b[i]) * b[i]);
    b2 = sqrt(b2);
    tol *= b2;
    lsgo_apply_c(op, sigma_im, x, r);
    for (i = 0; i < np; i++) r[i] = b[i] - r[i];
    t0 = now_s();
    while (r2 > tol && iter <= max_iter) {
        if (precond)
            for (i = 0; i < np; i++) r[i] /= diag;
        if (iter > 1) {
            const int k = (iter - 2) % m;
            for (i = 0; i < np; i++) {
                DX[k * np + i] = x[i] - x_old[i];
                DF[k * np + i] = r[i] - f_old[i];
            }
        }
        memcpy(x_old, x, sizeof(double complex) * np);
        memcpy(f_old, r, sizeof(double complex) * np);
        if (iter % p) {
            for (i = 0; i < np; i++) x[i] += omega * r[i];
        } else {
            const int m2 = 2 * m;
            for (int a = 0; a < m; a++)
                for (int j = 0; j <= a; j++) {
                    const double complex g = zdot(DF + a * np, DF + j * np, np); /* G(a,j) */
                    const double gre = creal(g), gim = (a == j) ? 0.0 : cimag(g);
                    /* real representation [[A, -B], [B, A]] of G = A + iB */
                    Gr[a * m2 + j] = gre;           Gr[j * m2 + a] = gre;
                    Gr[(a + m) * m2 + j + m] = gre; Gr[(j + m) * m2 + a + m] = gre;
                    Gr[a * m2 + j + m] = -gim;      Gr[j * m2 + a + m] = gim;
                    Gr[(a + m) * m2 + j] = gim;     Gr[(j + m) * m2 + a] = -gim;
                }
            for (int a = 0; a < m; a++) {
                const double complex h = zdot(DF + a * np, r, np);
                hr[a] = creal(h);
                hr[a + m] = cimag(h);
            }
            if (pinv_cut(Gr, hr, sr, m2, 2.22044605e-16)) status = 2;
            for (int a = 0; a < m; a++) {
                const double complex sa = sr[a] + I * sr[a + m];
                for (i = 0; i < np; i++) x[i] -= sa * (DX[a * np + i] + beta * DF[a * np + i]);
            }
            for (i = 0; i < np; i++) x[i] += beta * r[i];
        }
        lsgo_apply_c(op, sigma_im, x, r);
        for (i = 0; i < np; i++) r[i] = b[i] - r[i];
        if (iter % p == 0) {
            r2 = 0;
            for (i = 0; i < np; i++) r2 += creal(conj(r[i]) * r[i]);
            r2 = sqrt(r2);
        }
        iter++;
    }
    if (res) {
        res->seconds = now_s() - t0;
        res->iters = iter - 1;
        res->rhs_norm = b2;
        res->relres = r2 / b2;
        res->converged = r2 <= tol;
        res->status = status ? status : (res->converged ? 0 : 1);
    }
    free(r); free(x_old); free(f_old); free(DX); free(DF);
    return res ? res->status : 0;
}
