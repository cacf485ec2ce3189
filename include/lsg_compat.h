/*
 * lsg_compat.h — drop-in entry points with the reference's own prototypes.
 *
 * liblsg exports AAR, PGR, PL2R and CG exactly as YaphetS-jx/Linear-Solver
 * declares them, so MPI_REAL/main.c and system.c link against liblsg in
 * place of AAR.o, PGR.o, PL2R.o and CG.o, unchanged:
 *
 *   AAR   replaces MPI_REAL/AAR.c:37   (prototype MPI_REAL/AAR.h:18-22)
 *   PGR   replaces MPI_REAL/PGR.c:35   (prototype MPI_REAL/PGR.h:18-22)
 *   PL2R  replaces MPI_REAL/PL2R.c:35  (prototype MPI_REAL/PL2R.h:18-22)
 *   CG    replaces MPI_REAL/CG.c:33    (prototype MPI_REAL/CG.h:18-21)
 *
 * Behaviour kept from the reference: x (host, double[Np]) is the initial
 * guess on entry and the solution on exit; rhs is read only; tol is relative
 * to ||rhs||; the rank-0 report line ("AAR converged!:  Iterations = ...") is
 * printed in the reference's format.
 *
 * What changes: the operator and preconditioner run on the GPU, so the
 * host callbacks are not called.  The library recognises the reference's
 * Lap_Vec_mult / Precondition (the symbols of those names linked into the
 * process, or functions registered with lsg_register_operator_callback /
 * lsg_register_precondition_callback) and reads FDn, psize and coeff_lap
 * from the POISSON struct.  An unrecognised callback, a distributed domain
 * (psize != ssize, i.e. more than one MPI rank) or any failure leaves x
 * untouched, prints a one-line error to stderr and sets lsg_last_status().
 * There is no CPU fallback.
 *
 * Only the leading POISSON fields up to coeff_lap are read; their layout is
 * that of MPI_REAL/system.h:26-63 and does not depend on the MPI library
 * (the communicator members come after them).
 */
#ifndef LSG_COMPAT_H
#define LSG_COMPAT_H

#include "lsg.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifndef LSG_HAVE_POISSON
/* Layout of MPI_REAL/system.h:26-63 up to coeff_lap; the tail holds the
 * communicators, whose size depends on the MPI implementation. */
typedef struct lsg_poisson_prefix {
    int FDn;
    int ssize[3];
    int psize[3];
    int np[3];
    int coords[3];
    int rem[3];
    int *send_neighs;
    int *rec_neighs;
    int *send_counts;
    int *rec_counts;
    int send_layers[6];
    int rec_layers[6];
    int *scounts;
    int *sdispls;
    int *rcounts;
    int *rdispls;
    int n_in;
    int n_out;
    double *phi;
    double *rhs;
    double *Lap_phi;
    double solver_tol;
    int solver_maxiter;
    int m;
    int p;
    double omega;
    double beta;
    double *coeff_lap;
} POISSON;
typedef long lsg_comm_t; /* MPI_Comm: an int or a pointer, ignored by the library */
#define LSG_MPI_COMM lsg_comm_t
#else
#define LSG_MPI_COMM MPI_Comm
#endif

typedef void (*lsg_lap_fn)(POISSON *, double, double *, double *, LSG_MPI_COMM);
typedef void (*lsg_precond_fn)(double, double *, int);

void AAR(POISSON *system, lsg_lap_fn Lap_Vec_mult, lsg_precond_fn Precondition, double a,
         double *x, double *rhs, double omega, double beta, int m, int p, int max_iter,
         double tol, int Np, LSG_MPI_COMM comm);
void PGR(POISSON *system, lsg_lap_fn Lap_Vec_mult, lsg_precond_fn Precondition, double a,
         double *x, double *rhs, double omega, int m, int p, int max_iter, double tol, int Np,
         LSG_MPI_COMM comm);
void PL2R(POISSON *system, lsg_lap_fn Lap_Vec_mult, lsg_precond_fn Precondition, double a,
          double *x, double *rhs, double omega, int m, int p, int max_iter, double tol, int Np,
          LSG_MPI_COMM comm);
void CG(POISSON *system, lsg_lap_fn Lap_Vec_mult, lsg_precond_fn Precondition, double a,
        double *x, double *b, int max_iter, double tol, int Np, LSG_MPI_COMM comm);

/* Declare that `fn` computes the reference operator a*Lap*x of
 * MPI_REAL/system.c:80-213 (for callers whose Lap_Vec_mult has another name
 * or is not visible to dlsym).  Up to 8 registrations; returns lsg_status. */
int lsg_register_operator_callback(void *fn);
/* Declare that `fn` is the Jacobi division r[i] /= diag of system.c:222-227. */
/* Binds a user operator callback (a Lap_Vec_mult of the caller's own) to the
 * CSR form of its matrix (host arrays, copied to the device): the drop-in AAR
 * then solves with that matrix on the GPU, Jacobi from its diagonal when the
 * preconditioner is the reference one or registered.  Refused for PGR, PL2R
 * and CG.  The reference calls any operator through the callback
 * (MPI_REAL/README:25); a GPU solve needs the operator as data. */
int lsg_register_operator_csr(void *fn, int n, long long nnz, const int *row_ptr, const int *col,
                              const double *val);
int lsg_register_precondition_callback(void *fn);
/* Precision of the drop-in AAR: 0 (default) FP64 as the reference;
 * 1 mixed: FP32 inner AAR inside FP64 residual refinement, same tol on the
 * FP64 residual (iteration counts then differ from the reference's). */
void lsg_set_compat_mode(int mode);
/* Controls the reference-format report line: 1 print (default), 0 silent. */
void lsg_set_verbose(int on);
/* Result of the last AAR/PGR/PL2R/CG call on this thread. */
void lsg_last_result(lsg_result *res);

#ifdef __cplusplus
}
#endif
#endif /* LSG_COMPAT_H */
