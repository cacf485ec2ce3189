// lsg_kernels.cuh — the solver kernels, instantiated per vector type by
// lsg_kernels_f64.cu and lsg_kernels_f32.cu.
//
//   residual     r = b - A x  (+ AAR history column, ||r||^2)     system.c:80-213, AAR.c:119-123
//   richardson   fused x <- x + w D^-1 r ; r <- b - A x ; DX, DF  AAR.c:93-107,134-139; PGR.c:92-109
//   gram         Gram matrix of the history, FP64-class sums      AAR.c:192-210; PGR.c:188-204; PL2R.c:187-204
//   aar_update   Anderson extrapolation + history column           AAR.c:116-117, 225-231
//   proj_update  Galerkin / L2 projection + history fix-up         PGR.c:117-130; PL2R.c:115-129
//   cg_direction d = D^-1 r + beta d ; q = A d ; d.q               CG.c:94-100, 149-150
//   cg_step      x += alpha d ; r -= alpha q ; r.r                  CG.c:106-139
#pragma once

#include <algorithm>

#include "lsg_stencil.cuh"

namespace lsg {

constexpr int kReduceThreads = 256;

__device__ __forceinline__ bool solve_done(const DevCtrl *c) {
    return c != nullptr && *(volatile const int *)&c->done;
}

// ---------------------------------------------------------------- stencil functors

template <typename T, int MODE>
struct ResidualOp {
    static constexpr int NACC = (MODE == RES_APPLY) ? 0 : 1;
    const T *x;
    const T *b;
    T *r;
    T *df;
    T cf;
    double *partials;
    const DevCtrl *ctrl;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {}
    __device__ __forceinline__ T load(long long i) const { return ldg(x + i); }
    __device__ __forceinline__ void store(long long i, T u, T au, Acc<T> *acc) const {
        if (MODE == RES_APPLY) {
            r[i] = au;
        } else {
            const T rn = ldg(b + i) - au;
            if (MODE == RES_ANDERSON) df[i] = (rn - r[i]) * cf;
            r[i] = rn;
            acc[0].add_prod(rn, rn);
        }
    }
};

template <typename T, int MODE>
struct RichOp {
    static constexpr int NACC = 0;
    const T *x;
    const T *r;
    const T *b;
    T *x2;
    T *r2;
    T *dx;
    T *df;
    T c;   // omega * cf
    T cf;  // 1/diag (or 1 without preconditioning)
    double *partials;
    const DevCtrl *ctrl;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {}
    __device__ __forceinline__ T load(long long i) const { return fma(c, ldg(r + i), ldg(x + i)); }
    __device__ __forceinline__ void store(long long i, T u, T au, Acc<T> *) const {
        const T rn = ldg(b + i) - au;
        const T xo = ldg(x + i);
        const T ro = ldg(r + i);
        x2[i] = u;
        r2[i] = rn;
        dx[i] = u - xo;
        df[i] = (MODE == RICH_AAR) ? (rn - ro) * cf : (ro - rn);
    }
};

template <typename T>
struct CgDirOp {
    static constexpr int NACC = 1;
    const T *r;
    const T *d_old;
    T *d_new;
    T *q;
    T cf;
    T beta;
    double *partials;
    const DevCtrl *ctrl;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() { beta = (T)ctrl->beta; }
    __device__ __forceinline__ T load(long long i) const { return fma(beta, ldg(d_old + i), cf * ldg(r + i)); }
    __device__ __forceinline__ void store(long long i, T u, T au, Acc<T> *acc) const {
        d_new[i] = u;
        q[i] = au;
        acc[0].add_prod(u, au);
    }
};

struct IrResidualOp {
    static constexpr int NACC = 1;
    const double *x;
    const double *b;
    float *r32;
    double *partials;
    const DevCtrl *ctrl;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {}
    __device__ __forceinline__ double load(long long i) const { return ldg(x + i); }
    __device__ __forceinline__ void store(long long i, double u, double au, Acc<double> *acc) const {
        const double rn = ldg(b + i) - au;
        r32[i] = (float)rn;
        acc[0].add_prod(rn, rn);
    }
};

// ---------------------------------------------------------------- stencil dispatch

template <typename T, class Op>
cudaError_t launch_stencil(const StencilLaunch &L, const Weights<T> &w, const Op &op) {
    constexpr int BY = TileOf<T>::BY, NY = TileOf<T>::NY;
    const dim3 grid = stencil_grid(L.g, BY * NY, L.lz);
    const dim3 block(32, BY);
    if (w.radius == 6)
        stencil_kernel<T, 6, BY, NY, false, Op><<<grid, block, 0, L.stream>>>(L.g, w, L.lz, op);
    else
        stencil_kernel<T, LSG_MAX_RADIUS, BY, NY, true, Op><<<grid, block, 0, L.stream>>>(L.g, w, L.lz, op);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- point-local kernels

// Gram partials for history depth M (register accumulators).  FP32 vectors:
// products summed in FP32 over runs of kRun points, each run folded into a
// double-float accumulator; FP64 vectors: plain FP64 sums.
constexpr int kRun = 8;

template <typename T, int KIND, int M>
__global__ void __launch_bounds__(kReduceThreads) gram_kernel(const T *__restrict__ dx,
                                                              const T *__restrict__ df,
                                                              const T *__restrict__ r, long long n,
                                                              double *partials,
                                                              const DevCtrl *ctrl) {
    constexpr int NP = (KIND == GRAM_SYM) ? (M * (M + 1)) / 2 : M * M;
    constexpr int NV = NP + M;
    __shared__ double red[NV * (kReduceThreads / 32)];
    if (solve_done(ctrl)) return;
    Acc<T> acc[NV];
    T run[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) { acc[k].zero(); run[k] = T(0); }
    int cnt = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        T f[M], xv[KIND == GRAM_SYM ? 1 : M];
#pragma unroll
        for (int j = 0; j < M; j++) f[j] = ldg(df + j * n + i);
        if (KIND == GRAM_GALERKIN) {
#pragma unroll
            for (int j = 0; j < M; j++) xv[j] = ldg(dx + j * n + i);
        }
        const T rv = ldg(r + i);
        int k = 0;
        if (KIND == GRAM_SYM) {
#pragma unroll
            for (int j = 0; j < M; j++)
#pragma unroll
                for (int a = 0; a <= j; a++) { run[k] = fma(f[a], f[j], run[k]); k++; }
#pragma unroll
            for (int j = 0; j < M; j++) { run[NP + j] = fma(f[j], rv, run[NP + j]); }
        } else {
#pragma unroll
            for (int a = 0; a < M; a++)
#pragma unroll
                for (int j = 0; j < M; j++) { run[k] = fma(xv[a], f[j], run[k]); k++; }
#pragma unroll
            for (int j = 0; j < M; j++) { run[NP + j] = fma(xv[j], rv, run[NP + j]); }
        }
        if (sizeof(T) == 4 && ++cnt == kRun) {
#pragma unroll
            for (int q = 0; q < NV; q++) { acc[q].add(run[q]); run[q] = T(0); }
            cnt = 0;
        }
    }
    double v[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) { acc[q].add(run[q]); v[q] = acc[q].get(); }
    block_sum_store<NV>(v, red, partials + (long long)blockIdx.x * NV);
}

// Generic Gram (any m <= LSG_MAX_M): one value per (block, thread-slot), the
// history columns re-read per value from L2.  Used only for m > 8.
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) gram_generic_kernel(int kind, int m,
                                                                      const T *__restrict__ dx,
                                                                      const T *__restrict__ df,
                                                                      const T *__restrict__ r,
                                                                      long long n, int nv,
                                                                      double *partials,
                                                                      const DevCtrl *ctrl) {
    __shared__ double red[kReduceThreads / 32];
    if (solve_done(ctrl)) return;
    const int v = blockIdx.y;  // value index
    const int np = kind == GRAM_SYM ? (m * (m + 1)) / 2 : m * m;
    const T *u, *w;
    if (v < np) {
        if (kind == GRAM_SYM) {
            int j = 0;
            while ((j + 1) * (j + 2) / 2 <= v) j++;
            const int a = v - j * (j + 1) / 2;
            u = df + (long long)a * n; w = df + (long long)j * n;
        } else {
            const int a = v / m, j = v % m;
            u = dx + (long long)a * n; w = df + (long long)j * n;
        }
    } else {
        const int j = v - np;
        u = (kind == GRAM_SYM ? df : dx) + (long long)j * n; w = r;
    }
    Acc<T> acc;
    acc.zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        acc.add_prod(ldg(u + i), ldg(w + i));
    double s[1] = {acc.get()};
    double out;
    block_sum_store<1>(s, red, &out);
    if (threadIdx.x == 0) partials[(long long)blockIdx.x * nv + v] = out;
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) aar_update_kernel(int m, T *__restrict__ x,
                                                                    const T *__restrict__ r,
                                                                    T *__restrict__ dx,
                                                                    const T *__restrict__ df,
                                                                    int col, T beta, T cf,
                                                                    long long n,
                                                                    const DevCtrl *ctrl) {
    __shared__ T s[LSG_MAX_M];
    if (solve_done(ctrl)) return;
    if (threadIdx.x < m) s[threadIdx.x] = (T)ctrl->s[threadIdx.x];
    __syncthreads();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        T am = T(0);
        for (int j = 0; j < m; j++) am = fma(fma(beta, ldg(df + j * n + i), ldg(dx + j * n + i)), s[j], am);
        const T xo = x[i];
        const T xn = fma(beta, r[i] * cf, xo) - am;
        x[i] = xn;
        dx[(long long)col * n + i] = xn - xo;
    }
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) proj_update_kernel(int m, T *__restrict__ x,
                                                                     T *__restrict__ r,
                                                                     T *__restrict__ dx,
                                                                     T *__restrict__ df, int col,
                                                                     long long n,
                                                                     double *partials,
                                                                     const DevCtrl *ctrl) {
    __shared__ T s[LSG_MAX_M];
    __shared__ double red[kReduceThreads / 32];
    if (solve_done(ctrl)) return;
    if (threadIdx.x < m) s[threadIdx.x] = (T)ctrl->s[threadIdx.x];
    __syncthreads();
    Acc<T> acc;
    acc.zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        T tx = T(0), tf = T(0);
        for (int j = 0; j < m; j++) {
            tx = fma(ldg(dx + j * n + i), s[j], tx);
            tf = fma(ldg(df + j * n + i), s[j], tf);
        }
        x[i] += tx;
        const T rn = r[i] - tf;
        r[i] = rn;
        dx[(long long)col * n + i] += tx;
        df[(long long)col * n + i] += tf;
        acc.add_prod(rn, rn);
    }
    double v[1] = {acc.get()};
    block_sum_store<1>(v, red, partials + blockIdx.x);
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) cg_step_kernel(T *__restrict__ x,
                                                                 T *__restrict__ r,
                                                                 const T *__restrict__ d,
                                                                 const T *__restrict__ q,
                                                                 long long n, int restart,
                                                                 double *partials,
                                                                 const DevCtrl *ctrl) {
    __shared__ double red[kReduceThreads / 32];
    if (solve_done(ctrl)) return;
    const T alpha = (T)ctrl->alpha;
    Acc<T> acc;
    acc.zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        x[i] = fma(alpha, ldg(d + i), x[i]);
        if (!restart) {
            const T rn = fma(-alpha, ldg(q + i), r[i]);
            r[i] = rn;
            acc.add_prod(rn, rn);
        }
    }
    if (!restart) {
        double v[1] = {acc.get()};
        block_sum_store<1>(v, red, partials + blockIdx.x);
    }
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) norm2_kernel(const T *__restrict__ v, long long n,
                                                               double *partials,
                                                               const DevCtrl *ctrl) {
    __shared__ double red[kReduceThreads / 32];
    if (solve_done(ctrl)) return;
    Acc<T> acc;
    acc.zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T a = ldg(v + i);
        acc.add_prod(a, a);
    }
    double s[1] = {acc.get()};
    block_sum_store<1>(s, red, partials + blockIdx.x);
}

template <typename T>
__global__ void axpy_kernel(T *__restrict__ x, const T *__restrict__ y, T alpha, long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        x[i] = fma(alpha, y[i], x[i]);
}

// ---------------------------------------------------------------- host wrappers

template <typename T>
cudaError_t Kernels<T>::residual(const StencilLaunch &L, const Weights<T> &w, int mode,
                                 const T *x, const T *b, T *r, T *df, double cf,
                                 double *partials, const DevCtrl *ctrl) {
    switch (mode) {
    case RES_INIT: {
        ResidualOp<T, RES_INIT> op{x, b, r, df, (T)cf, partials, ctrl};
        return launch_stencil<T>(L, w, op);
    }
    case RES_ANDERSON: {
        ResidualOp<T, RES_ANDERSON> op{x, b, r, df, (T)cf, partials, ctrl};
        return launch_stencil<T>(L, w, op);
    }
    default: {
        ResidualOp<T, RES_APPLY> op{x, b, r, df, (T)cf, partials, ctrl};
        return launch_stencil<T>(L, w, op);
    }
    }
}

template <typename T>
cudaError_t Kernels<T>::richardson(const StencilLaunch &L, const Weights<T> &w, int mode,
                                   const T *x, const T *r, const T *b, T *x2, T *r2, T *dx,
                                   T *df, double c, double cf, const DevCtrl *ctrl) {
    if (mode == RICH_AAR) {
        RichOp<T, RICH_AAR> op{x, r, b, x2, r2, dx, df, (T)c, (T)cf, nullptr, ctrl};
        return launch_stencil<T>(L, w, op);
    }
    RichOp<T, RICH_PGR> op{x, r, b, x2, r2, dx, df, (T)c, (T)cf, nullptr, ctrl};
    return launch_stencil<T>(L, w, op);
}

template <typename T, int KIND>
static cudaError_t gram_dispatch(int m, const T *dx, const T *df, const T *r, long long n,
                                 double *partials, int blocks, const DevCtrl *ctrl,
                                 cudaStream_t s) {
    switch (m) {
#define LSG_GRAM_CASE(MM) \
    case MM: gram_kernel<T, KIND, MM><<<blocks, kReduceThreads, 0, s>>>(dx, df, r, n, partials, ctrl); break;
        LSG_GRAM_CASE(1) LSG_GRAM_CASE(2) LSG_GRAM_CASE(3) LSG_GRAM_CASE(4)
        LSG_GRAM_CASE(5) LSG_GRAM_CASE(6) LSG_GRAM_CASE(7) LSG_GRAM_CASE(8)
#undef LSG_GRAM_CASE
    default: {
        const int nv = gram_values(KIND, m);
        gram_generic_kernel<T><<<dim3(blocks, nv), kReduceThreads, 0, s>>>(KIND, m, dx, df, r, n, nv,
                                                                            partials, ctrl);
    }
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kernels<T>::gram(int kind, int m, const T *dx, const T *df, const T *r, long long n,
                             double *partials, int blocks, const DevCtrl *ctrl, cudaStream_t s) {
    if (kind == GRAM_SYM) return gram_dispatch<T, GRAM_SYM>(m, dx, df, r, n, partials, blocks, ctrl, s);
    return gram_dispatch<T, GRAM_GALERKIN>(m, dx, df, r, n, partials, blocks, ctrl, s);
}

template <typename T>
cudaError_t Kernels<T>::aar_update(int m, int col, T *x, const T *r, T *dx, const T *df,
                                   double beta, double cf, long long n, const DevCtrl *ctrl,
                                   cudaStream_t s) {
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, 152 * 8);
    aar_update_kernel<T><<<blocks, kReduceThreads, 0, s>>>(m, x, r, dx, df, col, (T)beta, (T)cf, n, ctrl);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kernels<T>::proj_update(int m, int col, T *x, T *r, T *dx, T *df, long long n,
                                    double *partials, int blocks, const DevCtrl *ctrl,
                                    cudaStream_t s) {
    proj_update_kernel<T><<<blocks, kReduceThreads, 0, s>>>(m, x, r, dx, df, col, n, partials, ctrl);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kernels<T>::cg_direction(const StencilLaunch &L, const Weights<T> &w, const T *r,
                                     const T *d_old, T *d_new, T *q, double cf, double *partials,
                                     const DevCtrl *ctrl) {
    CgDirOp<T> op{r, d_old, d_new, q, (T)cf, T(0), partials, ctrl};
    return launch_stencil<T>(L, w, op);
}

template <typename T>
cudaError_t Kernels<T>::cg_step(T *x, T *r, const T *d, const T *q, long long n, int restart,
                                double *partials, int blocks, const DevCtrl *ctrl,
                                cudaStream_t s) {
    cg_step_kernel<T><<<blocks, kReduceThreads, 0, s>>>(x, r, d, q, n, restart, partials, ctrl);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kernels<T>::norm2(const T *v, long long n, double *partials, int blocks,
                              const DevCtrl *ctrl, cudaStream_t s) {
    norm2_kernel<T><<<blocks, kReduceThreads, 0, s>>>(v, n, partials, ctrl);
    return cudaGetLastError();
}

template <typename T>
cudaError_t Kernels<T>::axpy(T *x, const T *y, double alpha, long long n, cudaStream_t s) {
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, 152 * 8);
    axpy_kernel<T><<<blocks, kReduceThreads, 0, s>>>(x, y, (T)alpha, n);
    return cudaGetLastError();
}

}  // namespace lsg
