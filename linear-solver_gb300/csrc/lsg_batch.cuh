// lsg_batch.cuh — batched kernels: one launch per pass covers every active
// instance of a batch (instances may differ in grid size, shift and
// coefficients).  Instantiated per vector type by lsg_batch_{f64,f32,c128,c64}.cu.
//
// A batched stencil launch is a 1-D grid: block b serves instance map[b],
// tile (b - sblk0) of that instance's (tx, ty, z-chunk) tile grid, with the
// same z-marching driver, functors and per-block partial sums as a single
// solve.  Point-local passes (Gram, extrapolation update, norms) give each
// instance `ublocks` grid-stride blocks.  The iteration number, the history
// column ((it-1) % m) and the residual ping-pong parity are computed on the
// device from the batch clock, so one captured cycle replays unchanged.
#pragma once

#include "lsg_kernels.cuh"

namespace lsg {

__device__ __forceinline__ int batch_iter(const BArgs &a) { return a.clk->it0 + a.k + 1; }

template <typename T>
__device__ __forceinline__ T *rbuf(const BInst<T> &I, int par) { return par ? I.r1 : I.r0; }
template <typename T>
__device__ __forceinline__ T *rbuf3(const BInst<T> &I, int k) { return k == 0 ? I.r0 : (k == 1 ? I.r1 : I.rs); }

// The residual after iterations 1..last: the ping-pong buffer, or (lean) the
// rotating one.
template <typename T>
__device__ __forceinline__ T *rcur(const BInst<T> &I, const BArgs &a, int last) {
    if (a.lean) {
        int s, c;
        lean_buffers(last, a.p, &s, &c);
        return rbuf3(I, c);
    }
    return rbuf(I, richardson_parity(last, a.p));
}


// Refinement passes act on instances whose FP32 iteration paused (gate 0), or
// on every unfinished one (gate 1, the final pass after max_iter).
__device__ __forceinline__ bool replace_gate(const BCtl &C, const BArgs &a) {
    if (solve_done(C.octrl)) return false;
    return a.gate == 1 || solve_done(C.ctrl);
}

// ---------------------------------------------------------------- passes
// make(): the functor of one instance for this launch, or false when the
// instance has nothing to do in it.

template <typename T>
struct PassRichRecur {  // AAR.c:93-107,134-139 in residual-recurrence form
    using TS = T;
    using Op = RichRecurOp<T>;
    static constexpr int MINB = 0;  // the tile variant's
    __device__ static bool make(const BInst<T> &I, const BCtl &C, const BArgs &a, Op &op) {
        const int it = batch_iter(a);
        if (it > a.max_iter) return false;
        const int rc = richardson_parity(it - 1, a.p);
        const long long off = (long long)((it - 1) % a.m) * I.g.n;
        op = Op{rbuf(I, rc), I.x, rbuf(I, rc ^ 1), I.dx + off, I.df + off, I.c, I.cf, T(a.beta), nullptr, C.ctrl};
        return true;
    }
    __device__ static Weights<TS> weights(const BInst<T> &I) { return I.w; }
};

template <typename T>
struct PassRichLean {  // the same step with x left out (rebuilt at the extrapolation)
    using TS = T;
    using Op = RichLeanOp<T>;
    static constexpr int MINB = 0;  // the tile variant's
    __device__ static bool make(const BInst<T> &I, const BCtl &C, const BArgs &a, Op &op) {
        const int it = batch_iter(a);
        if (it > a.max_iter) return false;
        int s, c;
        lean_buffers(it - 1, a.p, &s, &c);
        const long long off = (long long)((it - 1) % a.m) * I.g.n;
        op = Op{rbuf3(I, c), rbuf3(I, lean_target(s, c)), I.dx + off, I.df + off, I.c, I.cf, T(a.beta), nullptr,
                C.ctrl};
        return true;
    }
    __device__ static Weights<TS> weights(const BInst<T> &I) { return I.w; }
};

template <typename T>
struct PassRich {  // AAR.c:93-107,134-139, x and r ping-pong
    using TS = T;
    using Op = RichOp<T, RICH_AAR>;
    static constexpr int MINB = 0;  // the tile variant's
    __device__ static bool make(const BInst<T> &I, const BCtl &C, const BArgs &a, Op &op) {
        const int it = batch_iter(a);
        if (it > a.max_iter) return false;
        const int rc = richardson_parity(it - 1, a.p);
        const long long off = (long long)((it - 1) % a.m) * I.g.n;
        T *xo = rc ? I.xalt : I.x, *xn = rc ? I.x : I.xalt;
        op = Op{xo, rbuf(I, rc), I.b, xn, rbuf(I, rc ^ 1), I.dx + off, I.df + off, I.c, I.cf, T(a.beta),
                nullptr, C.ctrl};
        return true;
    }
    __device__ static Weights<TS> weights(const BInst<T> &I) { return I.w; }
};

template <typename T>
struct PassResInit {  // AAR.c:80-82
    using TS = T;
    using Op = ResidualOp<T, RES_INIT>;
    static constexpr int MINB = 0;  // the tile variant's
    __device__ static bool make(const BInst<T> &I, const BCtl &C, const BArgs &, Op &op) {
        op = Op{I.x, I.b, I.r0, nullptr, nullptr, I.cf, T(0.0), C.part, C.ctrl};
        return true;
    }
    __device__ static Weights<TS> weights(const BInst<T> &I) { return I.w; }
};

template <typename T>
struct PassResAnderson {  // AAR.c:116-123, reference form
    using TS = T;
    using Op = ResidualOp<T, RES_ANDERSON>;
    static constexpr int MINB = 0;  // the tile variant's
    __device__ static bool make(const BInst<T> &I, const BCtl &C, const BArgs &a, Op &op) {
        const int it = batch_iter(a);
        if (it > a.max_iter) return false;
        const int rc = richardson_parity(it - 1, a.p);
        const long long off = (long long)((it - 1) % a.m) * I.g.n;
        op = Op{rc ? I.xalt : I.x, I.b, rbuf(I, rc), I.df + off, I.dx + off, I.cf, T(a.beta), C.part, C.ctrl};
        return true;
    }
    __device__ static Weights<TS> weights(const BInst<T> &I) { return I.w; }
};

template <typename T>
struct PassResRecur {  // AAR.c:116-123, residual recurrence on the step in xalt
    using TS = T;
    using Op = ResRecurOp<T>;
    static constexpr int MINB = 0;  // the tile variant's
    __device__ static bool make(const BInst<T> &I, const BCtl &C, const BArgs &a, Op &op) {
        const int it = batch_iter(a);
        if (it > a.max_iter) return false;
        const long long off = (long long)((it - 1) % a.m) * I.g.n;
        op = Op{I.xalt, rcur(I, a, it - 1), I.df + off, I.dx + off, I.cf, T(a.beta), C.part, C.ctrl};
        return true;
    }
    __device__ static Weights<TS> weights(const BInst<T> &I) { return I.w; }
};

template <typename T>
struct PassIrResidual {  // r = float(b64 - A x64) after iteration it (mixed solves)
    using TS = typename WideOf<T>::type;
    using Op = IrResidualOp<TS, T>;
    static constexpr int MINB = 1;
    __device__ static bool make(const BInst<T> &I, const BCtl &C, const BArgs &a, Op &op) {
        if (!replace_gate(C, a)) return false;
        const int it = batch_iter(a);
        op = Op{I.x64, I.b64, rcur(I, a, it), C.part, C.octrl};
        return true;
    }
    __device__ static Weights<TS> weights(const BInst<T> &I) { return I.w64; }
};

// ---------------------------------------------------------------- kernels

// DFM: FP64 passes in double-float arithmetic (stencil_march_df).
template <typename T, int RQ, int BY, int NY, int MINB, bool GENERIC, class Pass, bool DFM = false>
__global__ void __launch_bounds__(32 * BY, MINB) batch_stencil_kernel(const BInst<T> *tab, BArgs a) {
    using TS = typename Pass::TS;
    constexpr int FX = 32 + 2 * RQ;
    constexpr int FY = BY * NY + 2 * RQ;
    __shared__ __align__(16) TS smem[2][FX * FY];
    const int i = a.map[blockIdx.x];
    const BCtl &C = a.ctl[i];
    const BInst<T> &I = tab[i];
    typename Pass::Op op;
    if (!Pass::make(I, C, a, op)) return;
    if (op.skip()) return;
    op.init();
    const int lb = blockIdx.x - C.sblk0;
    const int t = lb / I.tx;
    const Weights<TS> w = Pass::weights(I);
    if constexpr (DFM && IsDfMarch<TS>::value) {
        stencil_march_df<RQ, BY, NY, GENERIC>(I.g, w, I.lz, op, smem[0], smem[1], lb - t * I.tx, t % I.ty,
                                              t / I.ty, lb);
    } else {
        stencil_march<TS, RQ, BY, NY, GENERIC>(I.g, w, I.lz, op, smem[0], smem[1], lb - t * I.tx, t % I.ty,
                                               t / I.ty, lb);
    }
}

// The paired march (two columns per lane, 64-wide tiles) of one batched pass
// whose functor has one (the FP32 Richardson passes); a.map is the paired
// block map, the instance's paired tile grid is (ptx, pty) x z chunks of plz.
// Results equal the one-column march's bit for bit.
template <typename T, int BY, int NY, int MINB, class Pass>
__global__ void __launch_bounds__(32 * BY, MINB) batch_stencil_x2_kernel(const BInst<T> *tab, BArgs a) {
    constexpr int FX = 64 + 12;
    constexpr int FY = BY * NY + 12;
    __shared__ __align__(16) T smem[2][FX * FY];
    const int i = a.map[blockIdx.x];
    const BCtl &C = a.ctl[i];
    const BInst<T> &I = tab[i];
    typename Pass::Op op;
    if (!Pass::make(I, C, a, op)) return;
    if (op.skip()) return;
    op.init();
    const int lb = blockIdx.x - C.pblk0;
    const int t = lb / I.ptx;
    stencil_march_x2<T, BY, NY>(I.g, Pass::weights(I), I.plz, op, smem[0], smem[1], lb - t * I.ptx, t % I.pty,
                                t / I.pty, lb);
}

// Batched stencil tile: tile variant V of the vector type (the refinement
// pass keeps its own launch bounds); the generic-radius path uses variant 0
// with one row per thread (NY = 1) so the widest staged plane stays in 48 KB.
template <typename T, int V, bool GENERIC>
struct BTile {
    static constexpr int BY = GENERIC ? TileVar<T, 0>::BY : TileVar<T, V>::BY;
    static constexpr int NY = GENERIC ? 1 : TileVar<T, V>::NY;
    static constexpr int MINB = GENERIC ? 1 : TileVar<T, V>::MINB;
};

template <typename T, int V, class Pass>
cudaError_t launch_batch_var(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s) {
    using Tl = BTile<T, V, false>;
    constexpr int MB = Pass::MINB == 0 ? Tl::MINB : Pass::MINB;
    if constexpr (DfOk<typename Pass::Op>::value) {
        if (!a.exact) {
            batch_stencil_kernel<T, 6, Tl::BY, Tl::NY, MB, false, Pass, true><<<grid, dim3(32, Tl::BY), 0, s>>>(tab, a);
            return cudaGetLastError();
        }
    }
    batch_stencil_kernel<T, 6, Tl::BY, Tl::NY, MB, false, Pass><<<grid, dim3(32, Tl::BY), 0, s>>>(tab, a);
    return cudaGetLastError();
}

template <typename T, class Pass>
cudaError_t launch_batch_stencil(const BInst<T> *tab, const BArgs &a, int grid, bool generic, int var,
                                 cudaStream_t s) {
    if (grid <= 0) return cudaSuccess;
    if (!generic) {
        if (var == 1) return launch_batch_var<T, 1, Pass>(tab, a, grid, s);
        if (var == 2) return launch_batch_var<T, 2, Pass>(tab, a, grid, s);
        return launch_batch_var<T, 0, Pass>(tab, a, grid, s);
    }
    using Tl = BTile<T, 0, true>;
    if constexpr (DfOk<typename Pass::Op>::value) {
        if (!a.exact) {
            batch_stencil_kernel<T, LSG_MAX_RADIUS, Tl::BY, Tl::NY, 1, true, Pass, true>
                <<<grid, dim3(32, Tl::BY), 0, s>>>(tab, a);
            return cudaGetLastError();
        }
    }
    batch_stencil_kernel<T, LSG_MAX_RADIUS, Tl::BY, Tl::NY, 1, true, Pass><<<grid, dim3(32, Tl::BY), 0, s>>>(tab, a);
    return cudaGetLastError();
}

template <typename T, int M>
__global__ void __launch_bounds__(kReduceThreads) batch_gram_kernel(const BInst<T> *tab, BArgs a) {
    constexpr int NV = (M * (M + 1)) / 2 + M;
    const int i = a.map[blockIdx.x];
    const BCtl &C = a.ctl[i];
    const int it = batch_iter(a);
    if (it > a.max_iter || solve_done(C.ctrl)) return;
    const BInst<T> &I = tab[i];
    const T *r = rcur(I, a, it - 1);
    const long long lb = blockIdx.x - C.ublk0;
    if constexpr (IsCplx<T>::value) {
        gram_c_block<typename RealOf<T>::type, M>(I.df, r, I.g.n, C.part + lb * 2 * NV, lb, C.ublocks);
    } else {
        if (I.vec) gram_block<T, GRAM_SYM, M, true>(I.dx, I.df, r, I.g.n, C.part + lb * NV, lb, C.ublocks);
        else gram_block<T, GRAM_SYM, M, false>(I.dx, I.df, r, I.g.n, C.part + lb * NV, lb, C.ublocks);
    }
}

template <typename T, int M>
__global__ void __launch_bounds__(kReduceThreads) batch_update_kernel(const BInst<T> *tab, BArgs a) {
    const int i = a.map[blockIdx.x];
    const BCtl &C = a.ctl[i];
    const int it = batch_iter(a);
    if (it > a.max_iter || solve_done(C.ctrl)) return;
    const BInst<T> &I = tab[i];
    const long long lb = blockIdx.x - C.ublk0;
    if constexpr (IsRecur<T>::value) {
        if (a.lean) {  // x: the cycle-start iterate, rebuilt from the cycle's H columns
            int s, c;
            lean_buffers(it - 1, a.p, &s, &c);
            const unsigned mask = lean_mask(it - 1, a.p, a.m);
            if constexpr (!IsCplx<T>::value) {
                if (I.vec) {
                    aar_update_block<T, M, true, true>(a.m, I.x, rbuf3(I, c), I.dx, I.xalt, T(a.beta), I.cf, I.g.n,
                                                       C.ctrl, lb, C.ublocks, rbuf3(I, s), mask);
                    return;
                }
            }
            aar_update_block<T, M, false, true>(a.m, I.x, rbuf3(I, c), I.dx, I.xalt, T(a.beta), I.cf, I.g.n, C.ctrl,
                                                lb, C.ublocks, rbuf3(I, s), mask);
            return;
        }
    }
    const int rc = richardson_parity(it - 1, a.p);
    T *x, *step;
    if (IsRecur<T>::value) {
        x = I.x;
        step = I.xalt;  // the residual pass reads the step as its stencil input
    } else {
        x = rc ? I.xalt : I.x;
        step = I.dx + (long long)((it - 1) % a.m) * I.g.n;  // completed by the residual pass
    }
    if constexpr (!IsCplx<T>::value) {
        if (I.vec) {
            aar_update_block<T, M, true>(a.m, x, rbuf(I, rc), I.dx, step, T(a.beta), I.cf, I.g.n, C.ctrl, lb,
                                         C.ublocks);
            return;
        }
    }
    aar_update_block<T, M, false>(a.m, x, rbuf(I, rc), I.dx, step, T(a.beta), I.cf, I.g.n, C.ctrl, lb,
                                  C.ublocks);
}

// x += sum_mask H_j - beta cf (r - r_start) of instances still iterating at
// iteration it (a lean batch stopped by max_iter between extrapolations).
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) batch_fold_kernel(const BInst<T> *tab, BArgs a) {
    const int i = a.map[blockIdx.x];
    const BCtl &C = a.ctl[i];
    if (solve_done(C.ctrl) || solve_done(C.octrl)) return;
    const int it = batch_iter(a);
    const unsigned mask = lean_mask(it, a.p, a.m);
    if (mask == 0u) return;
    const BInst<T> &I = tab[i];
    int s, c;
    lean_buffers(it, a.p, &s, &c);
    const T *r = rbuf3(I, c), *rs = rbuf3(I, s);
    const long long n = I.g.n;
    const long long lb = blockIdx.x - C.ublk0;
    const long long stride = (long long)C.ublocks * blockDim.x;
    for (long long j = lb * blockDim.x + threadIdx.x; j < n; j += stride) {
        T ac = T(0);
        for (int q = 0; q < a.m; q++)
            if ((mask >> q) & 1u) ac = ac + ldg(I.dx + (long long)q * n + j);
        I.x[j] = I.x[j] + (ac - T(a.beta) * ((r[j] - rs[j]) * I.cf));
    }
}

// Constant-mode deflation of mixed batches: instances with a non-zero shift;
// which 1 only those being refined (the refinement passes' gate).
__device__ __forceinline__ bool deflate_gate(const BCtl &C, const BArgs &a, int which) {
    if (!(C.sig_re != 0.0 || C.sig_im != 0.0)) return false;
    return which == 0 || replace_gate(C, a);
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) batch_mean_sum_kernel(const BInst<T> *tab, BArgs a, int which) {
    using TW = typename WideOf<T>::type;
    __shared__ double red[2 * (kReduceThreads / 32)];
    const int i = a.map[blockIdx.x];
    const BCtl &C = a.ctl[i];
    if (!deflate_gate(C, a, which)) return;
    const BInst<T> &I = tab[i];
    const TW *v = which ? I.x64 : I.b64;
    double re = 0.0, im = 0.0;
    const long long lb = blockIdx.x - C.ublk0;
    const long long stride = (long long)C.ublocks * blockDim.x;
    for (long long j = lb * blockDim.x + threadIdx.x; j < I.g.n; j += stride) {
        if constexpr (IsCplx<TW>::value) {
            const TW u = v[j];
            re += u.x;
            im += u.y;
        } else {
            re += v[j];
        }
    }
    Acc<double> acc[2];
    acc[0].v = re;
    acc[1].v = im;
    block_reduce_store<2>(acc, red, C.part + 2 * lb);
}

// One block per active instance: the mean from its ublocks partials into
// octrl->bmean (which 0) or octrl->shift = bmean / sigma - mean (which 1).
static __global__ void batch_mean_finalize_kernel(BArgs a, const int *amap, int which) {
    __shared__ double red[2 * (kReduceThreads / 32)];
    __shared__ double out[2];
    const BCtl &C = a.ctl[amap[blockIdx.x]];
    if (!deflate_gate(C, a, which)) return;
    double re = 0.0, im = 0.0;
    for (int k = threadIdx.x; k < C.ublocks; k += blockDim.x) {
        re += C.part[2 * k];
        im += C.part[2 * k + 1];
    }
    Acc<double> acc[2];
    acc[0].v = re;
    acc[1].v = im;
    block_reduce_store<2>(acc, red, out);
    __syncthreads();
    if (threadIdx.x != 0) return;
    const double mr = out[0] / (double)C.n, mi = out[1] / (double)C.n;
    DevCtrl *o = C.octrl;
    if (which == 0) {
        o->bmean[0] = mr;
        o->bmean[1] = mi;
    } else {
        const double sr = C.sig_re, si = C.sig_im, d = sr * sr + si * si;
        o->shift[0] = (o->bmean[0] * sr + o->bmean[1] * si) / d - mr;
        o->shift[1] = (o->bmean[1] * sr - o->bmean[0] * si) / d - mi;
    }
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) batch_shift_kernel(const BInst<T> *tab, BArgs a) {
    using TW = typename WideOf<T>::type;
    const int i = a.map[blockIdx.x];
    const BCtl &C = a.ctl[i];
    if (!deflate_gate(C, a, 1)) return;
    const BInst<T> &I = tab[i];
    TW c;
    if constexpr (IsCplx<TW>::value) c = TW(C.octrl->shift[0], C.octrl->shift[1]);
    else c = C.octrl->shift[0];
    const long long lb = blockIdx.x - C.ublk0;
    const long long stride = (long long)C.ublocks * blockDim.x;
    for (long long j = lb * blockDim.x + threadIdx.x; j < I.g.n; j += stride) I.x64[j] = I.x64[j] + c;
}

template <typename T, bool WIDE>
__global__ void __launch_bounds__(kReduceThreads) batch_norm2_kernel(const BInst<T> *tab, BArgs a) {
    using TV = typename std::conditional<WIDE, typename WideOf<T>::type, T>::type;
    constexpr int W = AccWidth<TV>::value;
    __shared__ double red[(kReduceThreads / 32) * W];
    const int i = a.map[blockIdx.x];
    const BCtl &C = a.ctl[i];
    const BInst<T> &I = tab[i];
    const TV *v;
    if constexpr (WIDE) v = I.b64;
    else v = I.b;
    const long long lb = blockIdx.x - C.ublk0;
    Acc<TV> acc;
    acc.zero();
    const long long stride = (long long)C.ublocks * blockDim.x;
    for (long long j = lb * blockDim.x + threadIdx.x; j < I.g.n; j += stride) {
        const TV u = ldg(v + j);
        acc.add_prod(u, u);
    }
    Acc<TV> a1[1] = {acc};
    block_reduce_store<1>(a1, red, C.part + lb * W);
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) batch_ir_correct_kernel(const BInst<T> *tab, BArgs a) {
    using TW = typename WideOf<T>::type;
    const int i = a.map[blockIdx.x];
    const BCtl &C = a.ctl[i];
    if (!replace_gate(C, a)) return;
    const BInst<T> &I = tab[i];
    const long long lb = blockIdx.x - C.ublk0;
    const long long stride = (long long)C.ublocks * blockDim.x;
    TW *x = I.x64;
    T *e = I.x;
    for (long long j = lb * blockDim.x + threadIdx.x; j < I.g.n; j += stride) {
        x[j] += (TW)e[j];
        e[j] = T(0.0);
    }
}

// ---------------------------------------------------------------- launchers

template <typename T>
int BatchKernels<T>::tile_y(bool generic, int var) {
    if (generic) return BTile<T, 0, true>::BY * BTile<T, 0, true>::NY;
    return tile_var_rows<T>(var);
}

template <typename T, int V, bool GENERIC>
static int batch_rich_occupancy() {
    using P = typename std::conditional<IsRecur<T>::value, PassRichLean<T>, PassRich<T>>::type;
    using Tl = BTile<T, V, GENERIC>;
    int n = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &n, batch_stencil_kernel<T, GENERIC ? LSG_MAX_RADIUS : 6, Tl::BY, Tl::NY, Tl::MINB, GENERIC, P,
                                 DfOk<typename P::Op>::value>,
        32 * Tl::BY, 0);
    if (e != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    return n;
}

template <typename T>
int BatchKernels<T>::stencil_blocks_per_sm(bool generic, int var) {
    if (generic) return batch_rich_occupancy<T, 0, true>();
    if (var == 1) return batch_rich_occupancy<T, 1, false>();
    if (var == 2) return batch_rich_occupancy<T, 2, false>();
    return batch_rich_occupancy<T, 0, false>();
}

template <typename T>
cudaError_t BatchKernels<T>::richardson(const BInst<T> *tab, const BArgs &a, int grid, bool generic, int var,
                                        cudaStream_t s) {
    if constexpr (IsRecur<T>::value) {
        if (a.lean) return launch_batch_stencil<T, PassRichLean<T>>(tab, a, grid, generic, var, s);
        return launch_batch_stencil<T, PassRichRecur<T>>(tab, a, grid, generic, var, s);
    } else {
        return launch_batch_stencil<T, PassRich<T>>(tab, a, grid, generic, var, s);
    }
}

template <typename T>
cudaError_t BatchKernels<T>::richardson_paired(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        if (grid <= 0) return cudaSuccess;
        if (a.lean)
            batch_stencil_x2_kernel<T, kPairBY, kPairNY, kPairMINB, PassRichLean<T>>
                <<<grid, dim3(32, kPairBY), 0, s>>>(tab, a);
        else
            batch_stencil_x2_kernel<T, kPairBY, kPairNY, kPairMINB, PassRichRecur<T>>
                <<<grid, dim3(32, kPairBY), 0, s>>>(tab, a);
        return cudaGetLastError();
    } else {
        (void)tab, (void)a, (void)grid, (void)s;
        return cudaErrorInvalidValue;
    }
}

template <typename T>
int BatchKernels<T>::paired_blocks_per_sm() {
    if constexpr (std::is_same<T, float>::value) {
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &occ, batch_stencil_x2_kernel<T, kPairBY, kPairNY, kPairMINB, PassRichLean<T>>, 32 * kPairBY, 0) !=
                cudaSuccess ||
            occ < 1) {
            cudaGetLastError();
            occ = 1;
        }
        return occ;
    } else {
        return 0;
    }
}

template <typename T>
cudaError_t BatchKernels<T>::fold(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s) {
    if (grid <= 0) return cudaSuccess;
    if constexpr (IsRecur<T>::value) {
        if (!a.lean) return cudaSuccess;
        batch_fold_kernel<T><<<grid, kReduceThreads, 0, s>>>(tab, a);
        return cudaGetLastError();
    } else {
        return cudaSuccess;
    }
}

template <typename T>
cudaError_t BatchKernels<T>::residual_init(const BInst<T> *tab, const BArgs &a, int grid, bool generic, int var,
                                           cudaStream_t s) {
    return launch_batch_stencil<T, PassResInit<T>>(tab, a, grid, generic, var, s);
}

template <typename T>
cudaError_t BatchKernels<T>::residual_anderson(const BInst<T> *tab, const BArgs &a, int grid, bool generic,
                                               int var, cudaStream_t s) {
    if constexpr (IsRecur<T>::value) return launch_batch_stencil<T, PassResRecur<T>>(tab, a, grid, generic, var, s);
    else return launch_batch_stencil<T, PassResAnderson<T>>(tab, a, grid, generic, var, s);
}

template <typename T>
cudaError_t BatchKernels<T>::ir_residual(const BInst<T> *tab, const BArgs &a, int grid, bool generic, int var,
                                         cudaStream_t s) {
    if constexpr (IsRecur<T>::value)
        return launch_batch_stencil<T, PassIrResidual<T>>(tab, a, grid, generic, var, s);
    else return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t BatchKernels<T>::gram(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s) {
    if (grid <= 0) return cudaSuccess;
    switch (a.m) {
#define LSG_BGRAM(MM) case MM: batch_gram_kernel<T, MM><<<grid, kReduceThreads, 0, s>>>(tab, a); break;
        LSG_BGRAM(1) LSG_BGRAM(2) LSG_BGRAM(3) LSG_BGRAM(4) LSG_BGRAM(5) LSG_BGRAM(6) LSG_BGRAM(7) LSG_BGRAM(8)
#undef LSG_BGRAM
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t BatchKernels<T>::update(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s) {
    if (grid <= 0) return cudaSuccess;
    switch (a.m) {
#define LSG_BUPD(MM) case MM: batch_update_kernel<T, MM><<<grid, kReduceThreads, 0, s>>>(tab, a); break;
        LSG_BUPD(1) LSG_BUPD(2) LSG_BUPD(3) LSG_BUPD(4) LSG_BUPD(5) LSG_BUPD(6) LSG_BUPD(7) LSG_BUPD(8)
#undef LSG_BUPD
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t BatchKernels<T>::norm2_rhs(const BInst<T> *tab, const BArgs &a, int grid, bool wide, cudaStream_t s) {
    if (grid <= 0) return cudaSuccess;
    if (wide) batch_norm2_kernel<T, true><<<grid, kReduceThreads, 0, s>>>(tab, a);
    else batch_norm2_kernel<T, false><<<grid, kReduceThreads, 0, s>>>(tab, a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t BatchKernels<T>::mean_deflate(const BInst<T> *tab, const BArgs &au, int ugrid, const BArgs &aa,
                                          const int *amap, int nact, int which, cudaStream_t s) {
    if (ugrid <= 0 || nact <= 0) return cudaSuccess;
    if constexpr (IsRecur<T>::value) {
        batch_mean_sum_kernel<T><<<ugrid, kReduceThreads, 0, s>>>(tab, au, which);
        batch_mean_finalize_kernel<<<nact, kReduceThreads, 0, s>>>(aa, amap, which);
        if (which == 1) batch_shift_kernel<T><<<ugrid, kReduceThreads, 0, s>>>(tab, au);
        return cudaGetLastError();
    } else {
        (void)tab, (void)au, (void)aa, (void)amap, (void)which, (void)s;
        return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t BatchKernels<T>::ir_correct(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s) {
    if (grid <= 0) return cudaSuccess;
    if constexpr (IsRecur<T>::value) {
        batch_ir_correct_kernel<T><<<grid, kReduceThreads, 0, s>>>(tab, a);
        return cudaGetLastError();
    } else {
        return cudaErrorInvalidValue;
    }
}

}  // namespace lsg
