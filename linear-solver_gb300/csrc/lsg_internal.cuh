// lsg_internal.cuh — definitions shared by the liblsg kernels and host code.
//
// Device-resident solver state, reduction helpers and the kernel launch
// interface between the per-dtype kernel files and the host solver loops.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>
#include <string.h>

#include "../../include/lsg.h"
#include "lsg_complex.cuh"

namespace lsg {

// ----------------------------------------------------------------------------
// Device control block: one per workspace.  Kernels of a solve read `done`
// first and return at once when it is set, so the host can enqueue several
// extrapolation cycles ahead of its convergence read without changing the
// result (the iteration at which `done` was set is kept in `iters`).
struct DevCtrl {
    int done;         // 1: converged, failed or stopped -> later kernels are no-ops
    int status;       // lsg_status raised on the device (NaN, SVD sweep limit)
    int iters;        // reference iteration count at exit (AAR.c:153 reports iter-1)
    int restarts;     // mixed solves: FP32 runs started (outer control block only)
    double rhs_norm;  // ||b||
    double tol_abs;   // tol * ||b||  (AAR.c:79)
    double relres;    // last computed ||r|| (absolute)
    double alpha;     // CG step length
    double beta;      // CG direction update
    double delta;     // CG r.s
    double dq;        // CG d.q
    double best;      // smallest relres seen (stall detection of inner solves)
    int stall;        // checks since relres last fell below 0.7 * best
    int stall_limit;  // 0: off; else stop (done, stalled = 1) after this many checks
    int stalled;      // set when the stall rule ended the solve
    int svd_fallbacks;  // extrapolation steps whose Gram needed the Jacobi SVD
    double tol_frac;  // mixed solves (outer block): the next run's floor, as a fraction of tol_abs
    int floor_misses; // mixed solves (outer block): consecutive runs that reached the floor, true residual > tol
    int x_zero;       // mixed solves (outer block): the initial x64 was exactly zero
    int df_range;     // FP64 double-float stencil: a value beyond the float range was split
    double bmean[2];  // mixed solves (outer block): mean of b (re, im)
    double shift[2];  // mixed solves (outer block): constant added to x64 by the last deflation
    unsigned fin_ticket;  // Gram finalize: blocks done summing (0 between launches)
    double s[LSG_MAX_M];  // m x m solve output
};

// Mixed solves: the residual the next FP32 run stops at (absolute), from the
// true residual after a replacement and the FP32 residual the previous run
// paused at: a reduction rho, floored at tol_frac * tol_abs (tol_frac
// starting at 1).  The FP32 recurrence drifts from the true residual, so a
// run that reaches the tol floor can leave the true residual just above tol.
// One such miss is normal (the next run restarts from the exact residual and
// usually lands below tol); after two in a row the floor drops by the
// observed drift, with a factor 2 margin, instead of repeating itself.
// tol_frac and the miss count are per solve (the outer control block), so
// single and batched solves follow the same schedule.
__host__ __device__ inline double next_target(double *tol_frac, int *misses, double rho, double true_res,
                                              double fp32_res, double tol_abs, bool first) {
    if (!(*tol_frac > 0.0)) *tol_frac = 1.0;
    if (!first) {
        if (fp32_res <= *tol_frac * tol_abs && true_res > tol_abs && true_res > 0.0) {
            if (++*misses >= 2) {
                *tol_frac *= 0.5 * fp32_res / true_res;
                *misses = 0;
            }
        } else {
            *misses = 0;
        }
    }
    const double a = *tol_frac * tol_abs, b = rho * true_res;
    return a > b ? a : b;
}

// Geometry of one periodic grid.
struct Geom {
    int nx, ny, nz;
    long long nxy;
    long long n;
};

inline Geom make_geom(const int n[3]) {
    Geom g;
    g.nx = n[0]; g.ny = n[1]; g.nz = n[2];
    g.nxy = (long long)n[0] * n[1];
    g.n = g.nxy * n[2];
    return g;
}

// Host-side scalar of a vector type: double for real vectors, cplx<double>
// for complex ones (the complex shift, Jacobi factor and Anderson weights).
template <typename T> struct ScalarOf { using type = double; };
template <typename R> struct ScalarOf<cplx<R>> { using type = cplx<double>; };

// Stencil weights in the arithmetic type: w[0] = 3*a*c_0 + sigma (centre),
// w[p] = a*c_p.  Passed by value (kernel parameter space).
template <typename T>
struct Weights {
    T w[LSG_MAX_RADIUS + 1];
    int radius;
    // FP64 weights as three floats w = w1 + w2 + w3 (exactly: 72 >= 53 bits)
    // for the double-float march (complex128: the real parts; zero for the
    // other vector types)
    float wf[3 * (LSG_MAX_RADIUS + 1)];
    float wfi[3];  // complex128: the imaginary part of w[0] (the shift's), three floats
};

// Three floats whose sum is exactly the double w (each the float nearest the
// remainder left by the previous ones).
inline void split3(double w, float *out) {
    const float a = (float)w;
    const double r1 = w - (double)a;
    const float b = (float)r1;
    out[0] = a;
    out[1] = b;
    out[2] = (float)(r1 - (double)b);
}

// Host: weights and Jacobi factor of an operator in a vector type.
template <typename T>
inline Weights<T> make_weights(const lsg_operator *op) {
    Weights<T> w;
    memset(&w, 0, sizeof(w));
    w.radius = op->radius;
    if constexpr (IsCplx<T>::value) {
        w.w[0] = T(op->a * 3.0 * op->coeff[0] + op->sigma, op->sigma_im);
        for (int p = 1; p <= op->radius; p++) w.w[p] = T(op->a * op->coeff[p], 0.0);
        if constexpr (std::is_same<T, cplx<double>>::value) {
            for (int p = 0; p <= op->radius; p++) split3(w.w[p].x, w.wf + 3 * p);
            split3(w.w[0].y, w.wfi);
        }
    } else {
        w.w[0] = (T)(op->a * 3.0 * op->coeff[0] + op->sigma);
        for (int p = 1; p <= op->radius; p++) w.w[p] = (T)(op->a * op->coeff[p]);
        if constexpr (std::is_same<T, double>::value)
            for (int p = 0; p <= op->radius; p++) split3(w.w[p], w.wf + 3 * p);
    }
    return w;
}

// Re-derives the three-float weights after w.w changed.
template <typename T>
inline void refresh_df_weights(Weights<T> &w) {
    if constexpr (std::is_same<T, double>::value) {
        for (int p = 0; p <= LSG_MAX_RADIUS; p++) split3(w.w[p], w.wf + 3 * p);
    } else if constexpr (std::is_same<T, cplx<double>>::value) {
        for (int p = 0; p <= LSG_MAX_RADIUS; p++) split3(w.w[p].x, w.wf + 3 * p);
        split3(w.w[0].y, w.wfi);
    }
}

// Jacobi factor cf = 1 / diag (or 1 without preconditioning), in the
// vector type's host scalar: the complex shift makes it complex.
template <typename T>
inline typename ScalarOf<T>::type jacobi_factor(const lsg_operator *op) {
    if constexpr (IsCplx<T>::value) {
        if (!op->precond) return cplx<double>(1.0, 0.0);
        const double dr = op->a * (3 * op->coeff[0]) + op->sigma, di = op->sigma_im;
        const double den = dr * dr + di * di;
        return cplx<double>(dr / den, -di / den);
    } else {
        return op->precond ? 1.0 / (op->a * (3 * op->coeff[0]) + op->sigma) : 1.0;
    }
}

// Autotuned Richardson launch shape (lsg_tune.cu).
struct TuneEntry {
    int tile;          // tile variant
    int lz;            // z planes per block
    double us;         // measured time per launch
    double us_default; // the default shape's time
};
int tune_mode();
bool tune_lookup(int dtype, const Geom &g, TuneEntry *e);
struct StencilLaunch;
template <typename T>
StencilLaunch rich_launch(const lsg_operator *op, const StencilLaunch &L);

// Host helpers of lsg_solvers.cu.
int sm_count();
// 1: FP64 stencil passes in FP64 arithmetic (lsg_set_fp64_arith); 0: double-float.
int fp64_exact();
// The same for a solve to relative tolerance tol: the double-float sums leave
// a residual floor near 1e-13, so solves asking for less than kDfMinTol take
// the FP64-arithmetic march.
constexpr double kDfMinTol = 1e-10;
int fp64_exact_for(double tol);
// Form of the FP32 AAR's Richardson passes (lsg_set_aar_form): 0 ring, 1 lean, 2 x-carrying.
int aar_form();
int check_params(const lsg_params *prm, bool history);
// Initial control block: relres = tol + 1 (AAR.c:76), stall rule off (0) or on.
DevCtrl ctrl_init(double tol, int stall_limit);

// ----------------------------------------------------------------------------
// Reductions.  Every reducing kernel writes one partial per block (FP64) to a
// partials array; a finalize kernel sums them in a fixed order, so results
// are run-to-run deterministic.

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sums NV per-thread values over the block and writes them to out[0..NV) from
// thread 0.  `scratch` needs NV * (blockDim/32) doubles of shared memory.
template <int NV>
__device__ __forceinline__ void block_sum_store(double (&v)[NV], double *scratch, double *out) {
    const int lane = threadIdx.x & 31;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int warp = tid >> 5;
    const int nwarps = (blockDim.x * blockDim.y) >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double s = warp_sum(v[k]);
        if ((tid & 31) == 0) scratch[k * nwarps + warp] = s;
    }
    (void)lane;
    __syncthreads();
    if (tid < 32) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double s = tid < nwarps ? scratch[k * nwarps + tid] : 0.0;
            s = warp_sum(s);
            if (tid == 0) out[k] = s;
        }
    }
}

// Periodic index wrap valid for any integer v and n >= 1.
__host__ __device__ __forceinline__ int wrap_index(int v, int n) {
    int r = v % n;
    return r < 0 ? r + n : r;
}

// ----------------------------------------------------------------------------
// Kernel launch interface (implemented per dtype in lsg_kernels.cu).

enum ResidualMode {
    RES_INIT = 0,     // r = b - A x;                        acc ||r||^2
    RES_ANDERSON = 1, // r_new = b - A x; DF = (r_new-r)*cf; r = r_new;  acc ||r_new||^2
    RES_APPLY = 2,    // y = A x (no b, no reduction)
};

enum RichMode {
    RICH_AAR = 0,     // DF = (r_new - r) * cf   (difference of preconditioned residuals)
    RICH_PGR = 1,     // DF = r - r_new          (= A x_new - A x)
};

enum GramKind {
    GRAM_SYM = 0,     // G(i,j) = DF_i.DF_j (i <= j, symmetrised), h(j) = DF_j.r * hscale
    GRAM_GALERKIN = 1 // G(i,j) = DX_i.DF_j (all i,j), h(j) = DX_j.r * hscale
};

// The residual ring of the FP32 AAR.  The Richardson passes keep only the
// residual sequence: r_k (after iteration k) lives in ring slot k mod (m + 1),
// and history column k (written at iteration k, column (k - 1) mod m) is
//   DF_k = (r_k - r_{k-1}) cf,   H_k = c r_{k-1} + beta DF_k   (c = omega cf),
// rebuilt from two ring slots, with the arithmetic the x-carrying pass uses,
// wherever it is read.  Extrapolation columns (H_k = step + beta DF_k) keep H
// in the history array; a column whose r_k is later overwritten (the FP64
// residual replacement of a mixed solve) has DF (and H) stored first.
// RingWindow is one extrapolation's view: time t = 0..m-1 is the column of
// iteration k = it - m + t, column (s0 + t) mod m, read from slot[t] (r_{k-1})
// and slot[t + 1] (r_k); slot[m] holds the current residual r_{it-1}.
constexpr int kRingMaxM = 8;
struct RingWindow {
    int slot[kRingMaxM + 1];
    int s0;
    unsigned valid;  // bit t: the column exists (k >= 1)
    unsigned hmem;   // bit t: H stored in the history array
    unsigned dfmem;  // bit t: DF stored in the history array
    unsigned cyc;    // bit t: a Richardson step of the current cycle not yet added to x
    int e0, e1;      // times of the first two H-stored columns (-1: none)
};

struct StencilLaunch {
    Geom g;
    int lz;           // z planes per block
    cudaStream_t stream;
    int tile = 0;     // tile variant (passes without partial sums only)
    int paired = -1;  // 1: the two-columns-per-lane march (planned by Kernels<T>::paired_plan);
                      // 2: its 64 x 8 shape, 3: its 64 x 32 shape (passes without partial sums only);
                      // -1: the solver may choose it; 0: not
    int exact = 0;    // FP64 passes: 1 = FP64-arithmetic march, 0 = the double-float one
};

// Tile shape per vector type: FP64 is ALU-bound (narrower tile, fewer live
// registers); FP32 is bandwidth-bound (taller tile, less halo per point).
// A block is 32 x BY threads covering 32 x (BY*NY) columns.
template <typename T> struct TileOf;
template <> struct TileOf<double> { static constexpr int BY = 8, NY = 1, MINB = 2; };
template <> struct TileOf<float> { static constexpr int BY = 4, NY = 4, MINB = 4; };
template <> struct TileOf<cplx<double>> { static constexpr int BY = 8, NY = 1, MINB = 1; };
template <> struct TileOf<cplx<float>> { static constexpr int BY = 8, NY = 2, MINB = 2; };

// Tile variants the autotuner chooses from for the Richardson pass of single
// solves and for every stencil pass of a batch: (BY, NY, resident blocks the
// launch bounds ask for).  Variant 0 is TileOf<T>.
constexpr int kTileVariants = 3;
constexpr int kTilePaired = 3;  // tuner code of the two-columns-per-lane FP32 march
constexpr int kPairBY = 8, kPairNY = 2, kPairMINB = 2;  // its block: 32 x 8 threads, 64 x 16 tile
// A second shape of the paired march for the Richardson pass (tuner code 4):
// 32 x 4 threads, 64 x 8 tile, 4 blocks per SM.  Passes with a reduction
// keep the first shape (in the second they spill: 4 halo slots per thread).
constexpr int kTilePaired2 = 4;
constexpr int kPair2BY = 4, kPair2NY = 2, kPair2MINB = 4;
// A third, taller shape for passes without a reduction (tuner code 5): 32 x 8
// threads, 4 rows x 2 columns each (64 x 32 tile), one block per SM at ~210
// registers: ~0.56 staged halo values per point instead of 1.7 in 64 x 8.
constexpr int kTilePaired3 = 5;
constexpr int kPair3BY = 8, kPair3NY = 4, kPair3MINB = 1;
template <typename T, int V> struct TileVar;
template <> struct TileVar<double, 0> { static constexpr int BY = 8, NY = 1, MINB = 2; };
template <> struct TileVar<double, 1> { static constexpr int BY = 16, NY = 1, MINB = 1; };
// two rows per thread (32 x 16 tile, one 256-thread block per SM at ~200
// registers): ~26% fewer staged halo values per point, but half the warps to
// cover the FP64 epilogue's latency
template <> struct TileVar<double, 2> { static constexpr int BY = 8, NY = 2, MINB = 1; };
template <> struct TileVar<float, 0> { static constexpr int BY = 4, NY = 4, MINB = 4; };
template <> struct TileVar<float, 1> { static constexpr int BY = 8, NY = 2, MINB = 2; };
template <> struct TileVar<float, 2> { static constexpr int BY = 4, NY = 2, MINB = 4; };
template <> struct TileVar<cplx<double>, 0> { static constexpr int BY = 8, NY = 1, MINB = 1; };
template <> struct TileVar<cplx<double>, 1> { static constexpr int BY = 4, NY = 2, MINB = 1; };
template <> struct TileVar<cplx<double>, 2> { static constexpr int BY = 4, NY = 1, MINB = 2; };
template <> struct TileVar<cplx<float>, 0> { static constexpr int BY = 8, NY = 2, MINB = 2; };
template <> struct TileVar<cplx<float>, 1> { static constexpr int BY = 4, NY = 4, MINB = 2; };
template <> struct TileVar<cplx<float>, 2> { static constexpr int BY = 8, NY = 1, MINB = 2; };

// Rows (TY) of a tile variant.
template <typename T>
inline int tile_var_rows(int v) {
    switch (v) {
    case 1: return TileVar<T, 1>::BY * TileVar<T, 1>::NY;
    case 2: return TileVar<T, 2>::BY * TileVar<T, 2>::NY;
    default: return TileVar<T, 0>::BY * TileVar<T, 0>::NY;
    }
}

inline dim3 stencil_grid(const Geom &g, int ty, int lz) {
    return dim3((unsigned)((g.nx + 31) / 32), (unsigned)((g.ny + ty - 1) / ty),
                (unsigned)((g.nz + lz - 1) / lz));
}

// z planes per block, from a wave-balanced cost model: splitting each xy
// tile's column into c chunks gives bxy * c blocks, so a launch takes
// ceil(bxy c / slots) waves of blocks marching ceil(nz / c) planes each plus
// the 2R planes that refill the register queue of every chunk.  The refill
// weighs `fill` planes' worth of time: ~1 for bandwidth-bound passes (FP32,
// where it is reading), ~0.05 for FP64 (compute-bound: refilling is a few
// loads against ~44 FP64 operations per plane point).  Chunks stay >= 8 planes.
inline int balanced_lz(const Geom &g, int ty, int slots, double fill, int tw = 32) {
    const long long bxy = (long long)((g.nx + tw - 1) / tw) * ((g.ny + ty - 1) / ty);
    const int cmax = std::max(1, g.nz / 8);
    int best_lz = g.nz;
    double best = 1e300;
    for (int c = 1; c <= cmax; c++) {
        const int lz = (g.nz + c - 1) / c;
        const int cc = (g.nz + lz - 1) / lz;  // chunks actually used at this depth
        const long long waves = (bxy * cc + slots - 1) / slots;
        const double cost = (double)waves * (lz + fill * 12.0);
        if (cost < best - 1e-9) {
            best = cost;
            best_lz = lz;
        }
    }
    return std::max(1, std::min(best_lz, g.nz));
}

// Relative cost of a queue refill per vector type (see balanced_lz).
template <typename T> struct FillCost { static constexpr double value = 1.0; };
template <> struct FillCost<double> { static constexpr double value = 0.05; };
template <> struct FillCost<cplx<double>> { static constexpr double value = 0.05; };

template <typename T>
inline int choose_lz(const Geom &g, int slots) {
    return balanced_lz(g, TileOf<T>::BY * TileOf<T>::NY, slots, FillCost<T>::value);
}

// One-wave z depth for a tile of `ty` rows: as many chunks as fit in one wave.
inline int one_wave_lz(const Geom &g, int ty, int slots) {
    const long long bxy = (long long)((g.nx + 31) / 32) * ((g.ny + ty - 1) / ty);
    long long chunks = bxy >= slots ? 1 : slots / bxy;
    if (chunks < 1) chunks = 1;
    int lz = (int)((g.nz + chunks - 1) / chunks);
    if (lz < 8) lz = 8;
    if (lz > g.nz) lz = g.nz;
    return lz;
}

// Blocks (and so partial sums) of one stencil launch.
template <typename T>
inline long long stencil_blocks(const Geom &g, int lz) {
    const dim3 d = stencil_grid(g, TileOf<T>::BY * TileOf<T>::NY, lz);
    return (long long)d.x * d.y * d.z;
}

template <typename T>
struct Kernels {
    using S = typename ScalarOf<T>::type;
    // Resident blocks per SM of the fused Richardson stencil kernel (tile variant var).
    static int stencil_blocks_per_sm(int var = 0);
    // Paired (two columns per lane) march of the FP32 recurrence passes: its z
    // depth (*lz) and block count on grid g; 0 when T has none.
    static long long paired_plan(const Geom &g, int *lz);
    // Resident blocks per SM of paired shape 1 or 2 (0 when T has none).
    static int paired_blocks_per_sm(int shape);
    // y / r update driven by one stencil pass over x.  RES_ANDERSON also
    // completes the history column hc (holding x_new - x_old) with hb * DF_col.
    static cudaError_t residual(const StencilLaunch &L, const Weights<T> &w, int mode,
                                const T *x, const T *b, T *r, T *df, T *hc, S cf, double hb,
                                double *partials, const DevCtrl *ctrl);
    // Fused Richardson step: u = x + c*r at every stencil point; r2 = b - A u;
    // x2 = u; DF per mode; history column dx = (u - x) + hb * DF.
    static cudaError_t richardson(const StencilLaunch &L, const Weights<T> &w, int mode,
                                  const T *x, const T *r, const T *b, T *x2, T *r2, T *dx,
                                  T *df, S c, S cf, double hb, const DevCtrl *ctrl);
    // Residual-recurrence Richardson step (FP32 inner solver): r2 = r - c A r,
    // x += c r in place, DF = (r2 - r) cf, H = c r + hb DF.
    static cudaError_t richardson_recur(const StencilLaunch &L, const Weights<T> &w, const T *r,
                                        T *x, T *r2, T *dx, T *df, S c, S cf, double hb,
                                        const DevCtrl *ctrl);
    // The same step with x left out (r2, H, DF only); x is rebuilt by
    // aar_update_lean or recur_fold.
    static cudaError_t richardson_lean(const StencilLaunch &L, const Weights<T> &w, const T *r, T *r2,
                                       T *dx, T *df, S c, S cf, double hb, const DevCtrl *ctrl);
    // Extrapolation-step residual by recurrence: r -= A step; DF = (r_new - r) cf;
    // H_col = step + hb DF; ||r||^2.
    static cudaError_t residual_recur(const StencilLaunch &L, const Weights<T> &w, const T *step,
                                      T *r, T *df, T *hc, S cf, double hb, double *partials,
                                      const DevCtrl *ctrl);
    // ---- residual ring (FP32 only; other types return cudaErrorInvalidValue)
    // Richardson pass: r2 = r - c A r (nothing else is stored).
    static cudaError_t ring_richardson(const StencilLaunch &L, const Weights<T> &w, const T *r, T *r2, S c,
                                       const DevCtrl *ctrl);
    // Extrapolation-step residual: r2 = r - A step, H column hc = step + hb (r2 - r) cf, ||r2||^2.
    static cudaError_t ring_residual(const StencilLaunch &L, const Weights<T> &w, const T *step, const T *r,
                                     T *r2, T *hc, S cf, double hb, double *partials, const DevCtrl *ctrl);
    // Gram partials of the window's columns (column order, as gram() writes them).
    static cudaError_t ring_gram(int m, const RingWindow &rw, const T *ring, long long ss, const T *df, S cf,
                                 long long n, double *partials, int blocks, DevCtrl *ctrl, cudaStream_t s);
    // Extrapolation: x += the cycle's Richardson steps c r_{k-1} (in order),
    // step = beta cf r - sum_j H_j s_j, x += step.
    static cudaError_t ring_update(int m, const RingWindow &rw, const T *ring, long long ss, const T *h, T *x,
                                   T *step, S c, double beta, S cf, long long n, const DevCtrl *ctrl,
                                   cudaStream_t s);
    // x += the cycle's Richardson steps (a solve stopped between extrapolations).
    static cudaError_t ring_fold(int m, const RingWindow &rw, const T *ring, long long ss, T *x, S c, long long n,
                                 cudaStream_t s);
    // df = (rk - rk1) cf; h (if not null) = c rk1 + hb df.
    static cudaError_t ring_store_column(const T *rk1, const T *rk, T *df, T *h, S c, double hb, S cf,
                                         long long n, cudaStream_t s);
    // Paired-march z depth and block count of the ring passes (0 when T has none).
    static long long ring_paired_plan(const Geom &g, int *lz);
    // Grid of one Gram launch (one wave); partials written = grid * values.
    static int gram_grid(int kind, int m, long long n, int sms);
    // Gram partials over the history (point-local, grid-stride).  Complex
    // vectors: G(i,j) = DF_i^H DF_j, h_j = DF_j^H r (PETSC_COMPLEX/AAR_Complex.c:213-216).
    // exact = 0: FP64 vectors summed in double-float arithmetic (m <= 8).
    static cudaError_t gram(int kind, int m, const T *dx, const T *df, const T *r, long long n,
                            double *partials, int blocks, const DevCtrl *ctrl, cudaStream_t s, int exact = 1);
    // AAR extrapolation: x += beta*f - sum_j H_j s_j with f = r*cf and
    // H_j = DX_j + beta DF_j; step = x_new - x_old.
    static cudaError_t aar_update(int m, T *x, const T *r, const T *h, T *step, double beta,
                                  S cf, long long n, const DevCtrl *ctrl, cudaStream_t s);
    // The extrapolation after lean Richardson passes: x (the cycle-start
    // iterate) += sum_mask H_j - beta cf (r - rs) + step, step = beta cf r -
    // sum_j H_j s_j; rs is the cycle-start residual, bit j of mask marks the
    // cycle's Richardson columns.
    static cudaError_t aar_update_lean(int m, T *x, const T *r, const T *rs, const T *h, T *step,
                                       double beta, S cf, long long n, unsigned mask, const DevCtrl *ctrl,
                                       cudaStream_t s);
    // x += sum_mask H_j - beta cf (r - rs) (a lean solve stopped mid-cycle).
    static cudaError_t recur_fold(int m, T *x, const T *r, const T *rs, const T *h, double beta, S cf,
                                  long long n, unsigned mask, cudaStream_t s);
    // PGR/PL2R projection: tx = DX s, tf = DF s; x += tx; r -= tf; DX_col += tx;
    // DF_col += tf; partial ||r||^2.
    static cudaError_t proj_update(int m, int col, T *x, T *r, T *dx, T *df, long long n,
                                   double *partials, int blocks, const DevCtrl *ctrl,
                                   cudaStream_t s);
    // CG: d_new = r*cf + beta*d_old at every stencil point; q = A d_new; partial d.q.
    static cudaError_t cg_direction(const StencilLaunch &L, const Weights<T> &w, const T *r,
                                    const T *d_old, T *d_new, T *q, double cf,
                                    double *partials, const DevCtrl *ctrl);
    // CG: x += alpha d; r -= alpha q (restart=0) ; partials r.r (and r.s = cf*r.r).
    static cudaError_t cg_step(T *x, T *r, const T *d, const T *q, long long n, int restart,
                               double *partials, int blocks, const DevCtrl *ctrl,
                               cudaStream_t s);
    // partial ||v||^2 (grid-stride); complex vectors write (||v||^2, 0) pairs
    static cudaError_t norm2(const T *v, long long n, double *partials, int blocks,
                             const DevCtrl *ctrl, cudaStream_t s);
    // x += alpha*y  (alpha from the host)
    static cudaError_t axpy(T *x, const T *y, double alpha, long long n, cudaStream_t s);
};

// Mixed-precision helpers (lsg_kernels_f64.cu, lsg_kernels_c128.cu).
// r32 = float(b - A x64), partial ||b - A x64||^2 (FP64 stencil).
template <typename T64, typename T32>
cudaError_t ir_residual(const StencilLaunch &L, const Weights<T64> &w, const T64 *x,
                        const T64 *b, T32 *r32, double *partials, const DevCtrl *ctrl, int zgate = 0);
// The first refinement residual without the stencil when the initial x64
// was zero (ctrl->x_zero, set by zero_check): x64 is then the constant the
// deflation added (or 0), which A maps to sigma times itself, so
// r = b - sigma * shift.  It writes the partials of the stencil pass it
// replaces (`blocks` of them); ir_residual with zgate = 1 stands down then.
template <typename T64, typename T32>
cudaError_t ir_residual_const(const T64 *b, T32 *r32, long long n, double *partials, int blocks,
                              const DevCtrl *ctrl, double sig_re, double sig_im, cudaStream_t s);
// ctrl->x_zero = 0 when x holds a non-zero value (the host sets it to 1 first).
template <typename T64>
cudaError_t zero_check(const T64 *x, long long n, DevCtrl *ctrl, cudaStream_t s);
// x64 += e32; e32 = 0
template <typename T64, typename T32>
cudaError_t ir_correct(T64 *x, T32 *e, long long n, cudaStream_t s);
// Constant-mode deflation of mixed solves.  On the periodic grid the
// operator maps the constant vector to sigma times itself (the FD Laplacian's
// rows sum to zero), so the solution's mean is mean(b) / sigma exactly, and
// that mode -- the slowest one when sigma is small -- decouples.
// rhs_mean: ctrl->bmean = mean(b).  deflate_x: x += mean(b) / sigma -
// mean(x) (shift kept in ctrl->shift); the residual b - A x then has zero
// mean.  partials: >= 2 * reduce_blocks(n) doubles.
template <typename T64>
cudaError_t rhs_mean(const T64 *b, long long n, double *partials, DevCtrl *ctrl, cudaStream_t s);
template <typename T64>
cudaError_t deflate_x(T64 *x, long long n, double *partials, DevCtrl *ctrl, double sig_re, double sig_im,
                      cudaStream_t s);

// Finalize kernels (lsg_small.cu).
enum NormFinal {
    NF_RHS = 0,       // rhs_norm = sqrt(sum); tol_abs = tol * rhs_norm
    NF_CHECK = 1,     // relres = sqrt(sum); done if relres <= tol_abs (iters = iter)
    NF_STORE = 2,     // relres = sqrt(sum) only
};
// `width` = reals per partial (1 real, 2 complex: the norm is the real part).
cudaError_t finalize_norm(const double *partials, int nparts, DevCtrl *ctrl, int mode,
                          double tol, int iter, cudaStream_t s, int width = 1);
// Sums Gram partials, assembles G (m x m) and h (m), solves s = pinv(G) h with
// the reference semantics into ctrl->s.  hscale multiplies h.  Row 0 of the
// partials is overwritten with the totals.
cudaError_t finalize_gram_solve(double *partials, int nparts, int kind, int m, double hscale, DevCtrl *ctrl,
                                cudaStream_t s);
// Complex Hermitian variant: G(i,j) = DF_i^H DF_j, h = hscale * DF^H r; solved
// as its real 2m x 2m representation with zgelsd's cutoff (eps * sigma_max,
// PETSC_COMPLEX/AAR_Complex.c:239); ctrl->s holds (re, im) pairs, m <= 16.
cudaError_t finalize_gram_solve_c(double *partials, int nparts, int m, cplx<double> hscale, DevCtrl *ctrl,
                                  cudaStream_t s);
// CG scalars: mode 0: alpha = delta / sum(d.q).  mode 1: delta_new = cf*sum(r.r),
// relres = sqrt(sum r.r), beta = delta_new/delta_old, convergence test.
cudaError_t finalize_cg(const double *partials, int nparts, DevCtrl *ctrl, int mode, double cf,
                        int precond, int iter, int max_iter, cudaStream_t s);
cudaError_t pinv_solve_dev(const double *A, const double *b, double *x, int m, int *status,
                           cudaStream_t s);

// ----------------------------------------------------------------------------
// Batched solves (lsg_batch.cu).  All instances of a batch advance in
// lockstep through the same iteration numbers; every launch covers all active
// instances.  A block finds its instance through a block -> instance map and
// its share of the instance's work through the first-block / block-count
// fields of that instance's BCtl.  Finished instances are skipped through
// their DevCtrl flags, exactly as single solves skip queued work.

// FP32 vectors (real or complex) run AAR in residual-recurrence form.
template <typename T>
struct IsRecur { static constexpr bool value = std::is_same<typename RealOf<T>::type, float>::value; };

template <typename T> struct WideOf { using type = T; };
template <> struct WideOf<float> { using type = double; };
template <> struct WideOf<cplx<float>> { using type = cplx<double>; };

// Parity of the residual ping-pong after iterations 1..last (the Richardson
// iterations among them flip it; iteration 1 is one even when p = 1).
__host__ __device__ inline int richardson_parity(int last, int p) {
    if (last < 1) return 0;
    return (last - last / p + (p == 1 ? 1 : 0)) & 1;
}

// Lean FP32 AAR (Richardson passes leave x out): r rotates through three
// buffers.  A Richardson pass writes the buffer that is neither the current
// residual c nor the cycle-start residual s; the extrapolation residual is
// computed in place and starts the next cycle (s = c).  The buffers after
// iterations 1..last, in closed form: k complete cycles move s by
// 1 + ((p - 2) & 1) each; inside a cycle the passes alternate s+1, s+2.
__host__ __device__ inline void lean_buffers(int last, int p, int *s, int *c) {
    if (last < 1) { *s = 0; *c = 0; return; }
    if (p == 1) { *s = last == 1 ? 0 : 1; *c = 1; return; }  // iteration 1 is the only Richardson one
    const int k = last / p, rem = last % p;
    const int st = (int)(((long long)k * (1 + ((p - 2) & 1))) % 3);
    *s = st;
    *c = rem == 0 ? st : (st + 1 + ((rem - 1) & 1)) % 3;
}
// The buffer a Richardson pass writes, given s and c.
__host__ __device__ inline int lean_target(int s, int c) { return s == c ? (s + 1) % 3 : 3 - s - c; }
// History columns written by the Richardson passes since the last
// extrapolation, up to iteration `last` (bit (k-1) % m for iteration k).
__host__ __device__ inline unsigned lean_mask(int last, int p, int m) {
    unsigned mask = 0;
    for (int k = last; k >= 1 && !(k % p == 0 && k > 1); k--) mask |= 1u << ((k - 1) % m);
    return mask;
}

struct BClock {
    int it0;     // iterations covered by the cycles already run
    int ndone;   // finished instances (written by the cycle's last kernel)
    int pad[2];
};

// Type-independent part of an instance record.
struct BCtl {
    DevCtrl *ctrl;       // the AAR iteration (the FP32 one of a mixed solve)
    DevCtrl *octrl;      // mixed solves: the FP64 refinement; else nullptr
    double *part;        // this instance's partial sums
    long long n;
    int sblk0, sblocks;  // its share of the batched stencil launches
    int pblk0, pblocks;  // its share of the paired-march Richardson launches (FP32)
    int ublk0, ublocks;  // its share of the batched point-local launches
    double hre, him;     // scale of the Gram right-hand side (the Jacobi factor)
    double sig_re, sig_im;  // the operator's shift (mixed solves deflate the constant mode when non-zero)
};

template <typename T>
struct BInst {
    Geom g;
    int tx, ty, lz;      // stencil tiles along x and y; z planes per block
    int ptx, pty, plz;   // the same for the paired march (64-wide tiles; FP32 Richardson passes)
    int vec;             // n is a multiple of the 16-byte vector width
    Weights<T> w;
    Weights<typename WideOf<T>::type> w64;
    T cf, c;             // Jacobi factor, omega * cf
    T *x, *xalt, *r0, *r1, *dx, *df;
    T *rs;               // lean FP32: the third residual buffer
    const T *b;
    typename WideOf<T>::type *x64;        // mixed: the FP64 iterate and rhs
    const typename WideOf<T>::type *b64;
};

struct BArgs {
    const BCtl *ctl;
    const int *map;      // block -> instance
    const BClock *clk;
    int k;               // position in the cycle: iteration it = clk->it0 + k + 1
    int m, p, max_iter;
    double beta;
    int gate;            // refinement passes: 0 = paused instances, 1 = every unfinished one
    int lean;            // FP32: the Richardson passes leave x out (p - 1 <= m)
    int exact;           // FP64 stencil passes: 1 = FP64-arithmetic march (double-float otherwise)
};

template <typename T>
struct BatchKernels {
    // Resident blocks per SM of the batched Richardson pass in tile variant var.
    static int stencil_blocks_per_sm(bool generic, int var);
    // Tile height of the batched stencil passes in tile variant var.
    static int tile_y(bool generic, int var);
    // A lean batch stopped at max_iter between extrapolations: x += the
    // cycle's steps (unfinished instances; k as for the refinement passes).
    static cudaError_t fold(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s);
    // Richardson iteration k of the cycle (residual-recurrence form for FP32
    // vectors, the reference form for FP64 ones).
    static cudaError_t richardson(const BInst<T> *tab, const BArgs &a, int grid, bool generic, int var,
                                  cudaStream_t s);
    // The same pass in the paired march (FP32, radius 6, every nx even; a.map
    // is the paired block map); cudaErrorInvalidValue for other types.
    static cudaError_t richardson_paired(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s);
    // Resident blocks per SM of the paired Richardson pass (0 when T has none).
    static int paired_blocks_per_sm();
    // r0 = b - A x, ||r0||^2 partials.
    static cudaError_t residual_init(const BInst<T> *tab, const BArgs &a, int grid, bool generic, int var,
                                     cudaStream_t s);
    // The extrapolation iteration's residual, history column and ||r||^2.
    static cudaError_t residual_anderson(const BInst<T> *tab, const BArgs &a, int grid, bool generic, int var,
                                         cudaStream_t s);
    static cudaError_t gram(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s);
    static cudaError_t update(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s);
    // ||b||^2 partials (wide: the FP64 rhs of a mixed solve).
    static cudaError_t norm2_rhs(const BInst<T> *tab, const BArgs &a, int grid, bool wide, cudaStream_t s);
    // Mixed solves: r = float(b64 - A x64) into the current residual buffer.
    static cudaError_t ir_residual(const BInst<T> *tab, const BArgs &a, int grid, bool generic, int var,
                                   cudaStream_t s);
    // Mixed solves: x64 += e; e = 0.
    static cudaError_t ir_correct(const BInst<T> *tab, const BArgs &a, int grid, cudaStream_t s);
    // Constant-mode deflation of mixed batches (deflate_x for each instance
    // with a non-zero shift): which 0 stores mean(b64); 1 shifts x64 of the
    // instances being refined.  au: point-local map, aa + amap: one block per
    // active instance.  Three launches.
    static cudaError_t mean_deflate(const BInst<T> *tab, const BArgs &au, int ugrid, const BArgs &aa,
                                    const int *amap, int nact, int which, cudaStream_t s);
};

// Batched finalize kernels (lsg_small.cu): one block per active instance.
enum BatchFinal {
    BF_RHS = 0,          // ctrl: rhs norm from point-local partials
    BF_RHS_OUTER = 1,    // octrl: rhs norm from point-local partials
    BF_CHECK = 2,        // ctrl: convergence test after the extrapolation iteration
    BF_REPLACE = 3,      // octrl: FP64 residual norm of a refinement (gated)
};
cudaError_t batch_finalize_norm(const BArgs &a, const int *amap, int nact, int kind, double tol,
                                int width, cudaStream_t s);
cudaError_t batch_finalize_gram(const BArgs &a, const int *amap, int nact, bool complex_gram,
                                cudaStream_t s);
// Mixed solves: resume paused FP32 iterations (gated) with their next target.
cudaError_t batch_resume(const BArgs &a, const int *amap, int nact, double rho, int max_outer,
                         cudaStream_t s);
// it0 += p; ndone = finished instances; the int after the BClock of
// instance i = 1 if it finished.
cudaError_t batch_tick(BClock *clk, const BCtl *ctl, int count, int p, bool mixed, cudaStream_t s);

// ----------------------------------------------------------------------------
// General sparse operator (lsg_csr.cu): A in CSR form on the device, FP64.
struct CsrView {
    int n;
    long long nnz;
    const int *rp;      // n + 1 row offsets
    const int *col;     // nnz column indices
    const double *val;  // nnz values
    int group;          // lanes per row (4, 8, 16 or 32)
};
int csr_group(const CsrView &A);
cudaError_t csr_check(const CsrView &A, int phase, int *bad, int blocks, cudaStream_t s);
cudaError_t csr_diag(const CsrView &A, double *dinv, int precond, int *bad, int blocks, cudaStream_t s);
cudaError_t csr_residual(const CsrView &A, int mode, const double *x, const double *b, double *r, double *df,
                         double *hc, const double *dinv, double beta, double *partials, int blocks,
                         const DevCtrl *ctrl, cudaStream_t s);
cudaError_t csr_richardson(const CsrView &A, const double *x, const double *r, const double *b, double *x2,
                           double *r2, double *dx, double *df, const double *dinv, double omega, double beta,
                           int blocks, const DevCtrl *ctrl, cudaStream_t s);
cudaError_t csr_scale(const double *dinv, const double *r, double *f, long long n, int blocks,
                      const DevCtrl *ctrl, cudaStream_t s);

// Block-Jacobi ICC(0) (lsg_icc.cu): the factor of one (bx, by, bz) box of
// the operator (computed on the host, cached per device), its application
// f = M^-1 r fused with the AAR history completion (hist: DF = f - f_old,
// hc += beta DF), and the Richardson stencil pass with a materialised f
// (x2 = x + omega f, r2 = b - A x2, hn = omega f).
struct IccFactor;
int icc_factor_host(const int block[3], const double *w, int radius, double shift, double *L, double *d);
int icc_get(const lsg_operator *op, const int block[3], const IccFactor **out, double *shift);
cudaError_t icc_apply(const IccFactor *F, const Geom &g, const double *r, double *f, const double *f_old,
                      double *df, double *hc, double beta, int hist, const DevCtrl *ctrl, int exact, cudaStream_t s);
cudaError_t rich_prec(const StencilLaunch &L, const Weights<double> &w, const double *x, const double *f,
                      const double *b, double *x2, double *r2, double *hn, double omega, const DevCtrl *ctrl);

// Number of Gram values per block for a kind and history depth.
__host__ __device__ inline int gram_values(int kind, int m) {
    return kind == GRAM_SYM ? (m * (m + 1)) / 2 + m : m * m + m;
}

}  // namespace lsg
