// lsg_host.h — host-side internals shared by lsg_solvers.cu and lsg_compat.cpp.
#pragma once

#include <cuda_runtime.h>

#include "../../include/lsg.h"

namespace lsg {

int set_error(int status, const char *fmt, ...);
void set_last_status(int st);
int last_status();
const char *last_error();

// The reference FD coefficients c_0..c_radius (MPI_REAL/system.c:480-498).
int lap_coefficient(int radius, double *c);
int check_operator(const lsg_operator *op);
double jacobi_diag(const lsg_operator *op);

// solver: 0 AAR, 1 PGR, 2 PL2R, 3 CG
int solve(int solver, const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x,
          const void *d_b, lsg_result *res, cudaStream_t s);
int solve_mixed(const lsg_operator *op, const lsg_params *prm, double *x, const double *b,
                lsg_result *res, cudaStream_t s);
int solve_mixed_c(const lsg_operator *op, const lsg_params *prm, void *x, const void *b,
                  lsg_result *res, cudaStream_t s);
int apply(const lsg_operator *op, int dtype, const void *d_x, void *d_y, cudaStream_t s);
int pinv(const double *A, const double *b, double *x, int m, cudaStream_t s);
int release_workspaces();
// Batched AAR (lsg_batch.cu).
int solve_batched(const lsg_operator *ops, int count, const lsg_params *prm, int dtype, void *const *xs,
                  const void *const *bs, lsg_result *res, cudaStream_t s);
int solve_mixed_batched(const lsg_operator *ops, int count, const lsg_params *prm, int dtype, void *const *xs,
                        const void *const *bs, lsg_result *res, cudaStream_t s);
int release_batch_workspaces();
// General sparse operator (lsg_solvers.cu, kernels in lsg_csr.cu).
int solve_csr(const lsg_csr *A, const lsg_params *prm, double *x, const double *b, lsg_result *res,
              cudaStream_t s);
// Restarted GMRES (lsg_krylov.cu).
int gmres(const lsg_operator *op, const lsg_params *prm, int dtype, void *d_x, const void *d_b, lsg_result *res,
          cudaStream_t s, int aug = 0);
int release_gmres_workspaces();
// Block-Jacobi ICC(0) AAR (lsg_solvers.cu, kernels in lsg_icc.cu).
int solve_icc(const lsg_operator *op, const lsg_params *prm, const int block[3], double *x, const double *b,
              lsg_result *res, cudaStream_t s);
void release_icc();

}  // namespace lsg
