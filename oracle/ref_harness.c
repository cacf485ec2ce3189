/*
 * ref_harness.c — project-written entry points that drive the UNMODIFIED
 * reference solvers (YaphetS-jx/Linear-Solver MPI_REAL/*.c, compiled from
 * where they lie by oracle/Makefile against the one-rank MPI shim).
 *
 * Test infrastructure only: it is used in this container to pin the CPU
 * oracle (oracle/lsg_oracle.c) and to write the golden fixtures under
 * tests/golden/.  Nothing in the product links it.
 *
 * The reference solvers return nothing and report through printf on rank 0
 * (MPI_REAL/AAR.c:151-159, PGR.c:145-153, PL2R.c:144-152, CG.c:157-165), so
 * refh_solve() captures stdout around the call and parses that line.
 */
#include "system.h"
#include "AAR.h"
#include "PGR.h"
#include "PL2R.h"
#include "CG.h"
#include "tools.h"

#include <string.h>
#include <unistd.h>
#include <fcntl.h>

/* Builds the problem the way MPI_REAL/main.c:29-54 does for a one-rank world
 * and returns the reference's own right-hand side (system.c:452-468). */
int refh_rhs(int nx, int ny, int nz, int fdn, double *rhs_out)
{
    POISSON *s = calloc(1, sizeof(POISSON));
    int max_layer = 0, i, n;
    s->ssize[0] = nx; s->ssize[1] = ny; s->ssize[2] = nz; s->FDn = fdn;
    Processor_Domain(s->ssize, s->psize, s->np, s->coords, s->rem, MPI_COMM_WORLD, &s->cart);
    Max_layer(s->ssize, s->np, s->FDn, &max_layer);
    Initialize(s, max_layer);
    n = nx * ny * nz;
    for (i = 0; i < n; i++) rhs_out[i] = s->rhs[i];
    free(s->send_neighs); free(s->rec_neighs); free(s->send_counts); free(s->rec_counts);
    free(s->coeff_lap); free(s->phi); free(s->rhs); free(s->Lap_phi);
    free(s);
    return 0;
}

/* The reference FD coefficients (system.c:480-498). */
void refh_coefficients(int fdn, double *c)
{
    int i;
    for (i = 0; i <= fdn; i++) c[i] = 0.0;
    Lap_coefficient(c, fdn);
}

/* y = a * Lap * x with the reference's sequential operator (system.c:189-204). */
void refh_apply(int nx, int ny, int nz, int fdn, double a, double *x, double *y)
{
    POISSON s;
    memset(&s, 0, sizeof(s));
    s.FDn = fdn;
    s.psize[0] = s.ssize[0] = nx; s.psize[1] = s.ssize[1] = ny; s.psize[2] = s.ssize[2] = nz;
    s.coeff_lap = calloc(fdn + 1, sizeof(double));
    Lap_coefficient(s.coeff_lap, fdn);
    Lap_Vec_mult(&s, a, x, y, 1);
    free(s.coeff_lap);
}

/* x = PseudoInverseTimesVec(A, b) (tools.c:52-105); A row-major m x m. */
void refh_pinv(const double *A, const double *b, double *x, int m)
{
    double **rows = calloc(m, sizeof(double *));
    double *bb = calloc(m, sizeof(double));
    int i, j;
    for (i = 0; i < m; i++) {
        rows[i] = calloc(m, sizeof(double));
        for (j = 0; j < m; j++) rows[i][j] = A[i * m + j];
        bb[i] = b[i];
    }
    PseudoInverseTimesVec(rows, bb, x, m);
    for (i = 0; i < m; i++) free(rows[i]);
    free(rows);
    free(bb);
}

/* Runs one reference solver.  solver: 0 AAR, 1 PGR, 2 PL2R, 3 CG.
 * precond: 1 passes the reference Jacobi Precondition, 0 passes NULL.
 * x is overwritten with the solution.  Returns 0 when the report line was
 * found; *iters / *relres receive what the reference printed. */
int refh_solve(int solver, int nx, int ny, int nz, int fdn, double a, int precond,
               double *x, double *rhs, double omega, double beta, int m, int p,
               int max_iter, double tol, int *iters, double *relres, double *seconds)
{
    POISSON s;
    char path[] = "/tmp/refh_stdout_XXXXXX";
    char buf[4096];
    int fd, saved, got = -1, np = nx * ny * nz;
    ssize_t len;
    double t0, t1;
    void (*pc)(double, double *, int) = precond ? Precondition : NULL;

    memset(&s, 0, sizeof(s));
    s.FDn = fdn;
    s.psize[0] = s.ssize[0] = nx; s.psize[1] = s.ssize[1] = ny; s.psize[2] = s.ssize[2] = nz;
    s.coeff_lap = calloc(fdn + 1, sizeof(double));
    Lap_coefficient(s.coeff_lap, fdn);
    s.comm_laplacian = 3;

    fflush(stdout);
    fd = mkstemp(path);
    if (fd < 0) return -2;
    saved = dup(1);
    dup2(fd, 1);
    t0 = MPI_Wtime();
    switch (solver) {
    case 0: AAR(&s, Lap_Vec_mult, pc, a, x, rhs, omega, beta, m, p, max_iter, tol, np, 3); break;
    case 1: PGR(&s, Lap_Vec_mult, pc, a, x, rhs, omega, m, p, max_iter, tol, np, 3); break;
    case 2: PL2R(&s, Lap_Vec_mult, pc, a, x, rhs, omega, m, p, max_iter, tol, np, 3); break;
    default: CG(&s, Lap_Vec_mult, pc, a, x, rhs, max_iter, tol, np, 3); break;
    }
    t1 = MPI_Wtime();
    fflush(stdout);
    dup2(saved, 1);
    close(saved);
    lseek(fd, 0, SEEK_SET);
    len = read(fd, buf, sizeof(buf) - 1);
    close(fd);
    unlink(path);
    free(s.coeff_lap);
    if (seconds) *seconds = t1 - t0;
    if (len <= 0) return -1;
    buf[len] = 0;
    {
        const char *q = strstr(buf, "Iterations = ");
        if (q && sscanf(q, "Iterations = %d, Relative Residual = %lg", iters, relres) == 2) got = 0;
    }
    return got;
}
