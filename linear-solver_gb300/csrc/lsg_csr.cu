// lsg_csr.cu — kernels of the general sparse operator path: AAR on a
// user-supplied matrix A in CSR form (FP64) instead of the built-in stencil.
//
// The reference's AAR takes any operator through its Lap_Vec_mult callback
// (MPI_REAL/AAR.c:37, README:25); on the GPU the operator must be data, so the
// caller hands over the matrix.  Jacobi uses the matrix's own diagonal
// (D^-1, a vector here, a scalar for the stencil).  Rows are processed by
// groups of G lanes (G from the mean row length), each group reducing its
// row with warp shuffles (G = 1: a row per lane, so neighbouring rows'
// gathers of structured matrices coalesce); every warp iterates over the same
// row blocks, so the shuffles never see a lane that has left the loop.
//
//   csr_diag        D^-1 = 1 / a_ii (1 without preconditioning; zero diagonal flagged)
//   csr_residual    r = b - A x (+ ||r||^2); the extrapolation-step form also
//                   writes DF = D^-1 (r_new - r) and completes H = step + beta DF
//   csr_richardson  u = x + w D^-1 r gathered on the fly: x2 = u, r2 = b - A u,
//                   DF = D^-1 (r2 - r), H = (u - x) + beta DF     (AAR.c:93-107,134-139)
//   csr_scale       f = D^-1 r (the preconditioned residual of the extrapolation step)
#include "lsg_kernels.cuh"

namespace lsg {

template <int G>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o, G);
    return v;  // complete in lane 0 of the group
}

// Rows handled by this thread's group: row = base + lane / G, base advancing by
// whole warps, so the loop bounds are warp-uniform.
#define LSG_CSR_ROWS(G)                                                                      \
    const int lane_ = threadIdx.x & 31, sub_ = lane_ % (G);                                  \
    const long long warp_ = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;         \
    const long long nwarps_ = ((long long)gridDim.x * blockDim.x) >> 5;                      \
    constexpr int RPW_ = 32 / (G);                                                           \
    for (long long base_ = warp_ * RPW_; base_ < n; base_ += nwarps_ * RPW_)

template <int G>
__global__ void __launch_bounds__(kReduceThreads) csr_diag_kernel(int n, const int *__restrict__ rp,
                                                                  const int *__restrict__ col,
                                                                  const double *__restrict__ val,
                                                                  double *dinv, int precond, int *bad) {
    LSG_CSR_ROWS(G) {
        const long long row = base_ + lane_ / G;
        double d = 0.0;
        if (row < n)
            for (int k = rp[row] + sub_; k < rp[row + 1]; k += G)
                if (col[k] == row) d += val[k];
        d = group_sum<G>(d);
        if (row < n && sub_ == 0) {
            if (precond && d == 0.0) atomicExch(bad, 1);
            dinv[row] = (precond && d != 0.0) ? 1.0 / d : 1.0;
        }
    }
}

template <int G, int MODE>
__global__ void __launch_bounds__(kReduceThreads) csr_residual_kernel(
    int n, const int *__restrict__ rp, const int *__restrict__ col, const double *__restrict__ val,
    const double *__restrict__ x, const double *__restrict__ b, double *r, double *df, double *hc,
    const double *__restrict__ dinv, double beta, double *partials, const DevCtrl *ctrl) {
    __shared__ double red[kReduceThreads / 32];
    if (solve_done(ctrl)) return;
    Acc<double> acc;
    acc.zero();
    LSG_CSR_ROWS(G) {
        const long long row = base_ + lane_ / G;
        double s = 0.0;
        if (row < n)
            for (int k = rp[row] + sub_; k < rp[row + 1]; k += G) s = fma(val[k], ldg(x + col[k]), s);
        s = group_sum<G>(s);
        if (row < n && sub_ == 0) {
            if (MODE == RES_APPLY) {
                r[row] = s;
            } else {
                const double rn = b[row] - s;
                if (MODE == RES_ANDERSON) {
                    const double dfv = dinv[row] * (rn - r[row]);
                    df[row] = dfv;
                    hc[row] = fma(beta, dfv, hc[row]);
                }
                r[row] = rn;
                acc.add_prod(rn, rn);
            }
        }
    }
    if (MODE != RES_APPLY) {
        Acc<double> a1[1] = {acc};
        block_reduce_store<1>(a1, red, partials + blockIdx.x);
    }
}

template <int G>
__global__ void __launch_bounds__(kReduceThreads) csr_richardson_kernel(
    int n, const int *__restrict__ rp, const int *__restrict__ col, const double *__restrict__ val,
    const double *__restrict__ x, const double *__restrict__ r, const double *__restrict__ b,
    double *__restrict__ x2, double *__restrict__ r2, double *__restrict__ dx, double *__restrict__ df,
    const double *__restrict__ dinv, double omega, double beta, const DevCtrl *ctrl) {
    if (solve_done(ctrl)) return;
    LSG_CSR_ROWS(G) {
        const long long row = base_ + lane_ / G;
        double s = 0.0;
        if (row < n)
            for (int k = rp[row] + sub_; k < rp[row + 1]; k += G) {
                const int c = col[k];
                s = fma(val[k], fma(omega * ldg(dinv + c), ldg(r + c), ldg(x + c)), s);
            }
        s = group_sum<G>(s);
        if (row < n && sub_ == 0) {
            const double xo = x[row], ro = r[row], di = dinv[row];
            const double u = fma(omega * di, ro, xo);
            const double rn = b[row] - s;
            const double dfv = di * (rn - ro);
            x2[row] = u;
            r2[row] = rn;
            dx[row] = fma(beta, dfv, u - xo);
            df[row] = dfv;
        }
    }
}

__global__ void __launch_bounds__(kReduceThreads) csr_scale_kernel(const double *__restrict__ dinv,
                                                                   const double *__restrict__ r, double *f,
                                                                   long long n, const DevCtrl *ctrl) {
    if (solve_done(ctrl)) return;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) f[i] = dinv[i] * r[i];
}

#undef LSG_CSR_ROWS

// Structure checks of a caller's matrix, run before any gather: phase 0 reads
// only rp[0..n] (rp[0] = 0, non-decreasing, rp[n] = nnz); phase 1, run only
// when phase 0 passed, reads only col[0..nnz) (0 <= col < n).  A failure sets
// *bad; nothing is read outside the ranges the caller declared.
__global__ void csr_check_kernel(int n, long long nnz, const int *__restrict__ rp, const int *__restrict__ col,
                                 int phase, int *bad) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (phase == 0) {
        if (t0 == 0 && (rp[0] != 0 || (long long)rp[n] != nnz)) atomicExch(bad, 1);
        for (long long i = t0; i < n; i += stride)
            if (rp[i + 1] < rp[i]) atomicExch(bad, 1);
    } else {
        for (long long k = t0; k < nnz; k += stride)
            if (col[k] < 0 || col[k] >= n) atomicExch(bad, 1);
    }
}

cudaError_t csr_check(const CsrView &A, int phase, int *bad, int blocks, cudaStream_t s) {
    csr_check_kernel<<<blocks, kReduceThreads, 0, s>>>(A.n, A.nnz, A.rp, A.col, phase, bad);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- launchers

int csr_group(const CsrView &A) {
    const double mean = A.n > 0 ? (double)A.nnz / (double)A.n : 1.0;
    // measured on 128^3 matrices (7 and 37 entries per row): a row per lane
    // is 2x faster than any group; long rows need lanes to share the row
    return mean <= 48 ? 1 : mean <= 128 ? 8 : 32;
}

cudaError_t csr_diag(const CsrView &A, double *dinv, int precond, int *bad, int blocks, cudaStream_t s) {
    switch (A.group) {
    case 1: csr_diag_kernel<1><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, dinv, precond, bad); break;
    case 4: csr_diag_kernel<4><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, dinv, precond, bad); break;
    case 8: csr_diag_kernel<8><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, dinv, precond, bad); break;
    case 16: csr_diag_kernel<16><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, dinv, precond, bad); break;
    default: csr_diag_kernel<32><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, dinv, precond, bad);
    }
    return cudaGetLastError();
}

template <int MODE>
static void csr_residual_mode(const CsrView &A, const double *x, const double *b, double *r, double *df,
                              double *hc, const double *dinv, double beta, double *partials, int blocks,
                              const DevCtrl *ctrl, cudaStream_t s) {
    switch (A.group) {
    case 1:
        csr_residual_kernel<1, MODE><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, x, b, r, df, hc,
                                                                      dinv, beta, partials, ctrl);
        break;
    case 4:
        csr_residual_kernel<4, MODE><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, x, b, r, df, hc,
                                                                      dinv, beta, partials, ctrl);
        break;
    case 8:
        csr_residual_kernel<8, MODE><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, x, b, r, df, hc,
                                                                      dinv, beta, partials, ctrl);
        break;
    case 16:
        csr_residual_kernel<16, MODE><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, x, b, r, df, hc,
                                                                       dinv, beta, partials, ctrl);
        break;
    default:
        csr_residual_kernel<32, MODE><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, x, b, r, df, hc,
                                                                       dinv, beta, partials, ctrl);
    }
}

cudaError_t csr_residual(const CsrView &A, int mode, const double *x, const double *b, double *r, double *df,
                         double *hc, const double *dinv, double beta, double *partials, int blocks,
                         const DevCtrl *ctrl, cudaStream_t s) {
    if (mode == RES_INIT) csr_residual_mode<RES_INIT>(A, x, b, r, df, hc, dinv, beta, partials, blocks, ctrl, s);
    else if (mode == RES_ANDERSON)
        csr_residual_mode<RES_ANDERSON>(A, x, b, r, df, hc, dinv, beta, partials, blocks, ctrl, s);
    else csr_residual_mode<RES_APPLY>(A, x, b, r, df, hc, dinv, beta, partials, blocks, ctrl, s);
    return cudaGetLastError();
}

cudaError_t csr_richardson(const CsrView &A, const double *x, const double *r, const double *b, double *x2,
                           double *r2, double *dx, double *df, const double *dinv, double omega, double beta,
                           int blocks, const DevCtrl *ctrl, cudaStream_t s) {
    switch (A.group) {
    case 1:
        csr_richardson_kernel<1><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, x, r, b, x2, r2, dx, df,
                                                                   dinv, omega, beta, ctrl);
        break;
    case 4:
        csr_richardson_kernel<4><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, x, r, b, x2, r2, dx, df,
                                                                   dinv, omega, beta, ctrl);
        break;
    case 8:
        csr_richardson_kernel<8><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, x, r, b, x2, r2, dx, df,
                                                                   dinv, omega, beta, ctrl);
        break;
    case 16:
        csr_richardson_kernel<16><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, x, r, b, x2, r2, dx,
                                                                    df, dinv, omega, beta, ctrl);
        break;
    default:
        csr_richardson_kernel<32><<<blocks, kReduceThreads, 0, s>>>(A.n, A.rp, A.col, A.val, x, r, b, x2, r2, dx,
                                                                    df, dinv, omega, beta, ctrl);
    }
    return cudaGetLastError();
}

cudaError_t csr_scale(const double *dinv, const double *r, double *f, long long n, int blocks,
                      const DevCtrl *ctrl, cudaStream_t s) {
    csr_scale_kernel<<<blocks, kReduceThreads, 0, s>>>(dinv, r, f, n, ctrl);
    return cudaGetLastError();
}

}  // namespace lsg
