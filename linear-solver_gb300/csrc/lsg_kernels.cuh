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
#include <cstdlib>
#include <type_traits>

#include "lsg_stencil.cuh"

namespace lsg {

constexpr int kReduceThreads = 256;

__device__ __forceinline__ bool solve_done(const DevCtrl *c) {
    return c != nullptr && *(volatile const int *)&c->done;
}

// j-th extrapolation coefficient from the m x m solve (complex: (re, im) pairs).
template <typename T>
__device__ __forceinline__ T ctrl_s(const DevCtrl *c, int j) {
    if constexpr (IsCplx<T>::value) {
        using R = typename RealOf<T>::type;
        return T((R)c->s[2 * j], (R)c->s[2 * j + 1]);
    } else {
        return (T)c->s[j];
    }
}

// ---------------------------------------------------------------- stencil functors

template <typename T> struct Pair { T a, b; };
template <typename T> struct Triple { T a, b, c; };

// r = b - A x (RES_INIT, with ||r||^2), the AAR extrapolation residual
// (RES_ANDERSON: also DF_col = (r_new - r) cf, r in place, and the history
// column H_col, which holds the step x_new - x_old, completed to
// x_new - x_old + beta DF_col), or y = A x.
template <typename T, int MODE>
struct ResidualOp {
    static constexpr int NACC = (MODE == RES_APPLY) ? 0 : 1;
    // FP64 solves evaluate the sums in double-float; y = A x (lsg_apply, used
    // to check results) keeps FP64 arithmetic
    static constexpr bool DF = std::is_same<T, double>::value && MODE != RES_APPLY;
    using Raw = T;
    using Ctr = typename std::conditional<MODE == RES_ANDERSON, Triple<T>,
                typename std::conditional<MODE == RES_INIT, T, NoCtr>::type>::type;
    const T *x;
    const T *b;
    T *r;
    T *df;
    T *hc;
    T cf;
    T hb;
    double *partials;
    const DevCtrl *ctrl;
    float2 cfp;  // cf as a double-float pair (double-float march)
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {
        if constexpr (DF) cfp = df_weight((double)cf);
    }
    __device__ __forceinline__ Raw fetch(unsigned i) const { return ldg(x + i); }
    __device__ __forceinline__ T value(const Raw &v) const { return v; }
    __device__ __forceinline__ Ctr fetch_center(unsigned i) const {
        if constexpr (MODE == RES_ANDERSON) return Ctr{ldg(b + i), r[i], hc[i]};
        else if constexpr (MODE == RES_INIT) return ldg(b + i);
        else return Ctr{};
    }
    // Double-float epilogue: A u rounded to a double once, then the FP64
    // epilogue of store() (a few FP64 operations instead of double-float ones).
    static constexpr bool STORE_DF = DF;
    __device__ __forceinline__ void store_df(unsigned i, float2, float2 au, const Ctr &c, int k,
                                             Acc<T> *acc) const {
        store(i, T(0), (T)df_to_double(au, k), c, acc);
    }
    __device__ __forceinline__ void store(unsigned i, T u, T au, const Ctr &c, Acc<T> *acc) const {
        if constexpr (MODE == RES_APPLY) {
            r[i] = au;
        } else if constexpr (MODE == RES_INIT) {
            const T rn = c - au;
            r[i] = rn;
            acc[0].add_prod(rn, rn);
        } else {
            const T rn = c.a - au;
            const T dfv = (rn - c.b) * cf;
            df[i] = dfv;
            hc[i] = fma(hb, dfv, c.c);
            r[i] = rn;
            acc[0].add_prod(rn, rn);
        }
    }
};

// Fused Richardson step in the reference's form (AAR.c:93-107,134-139;
// PGR.c:92-109): u = x + omega*cf*r at every stencil point, r2 = b - A u,
// x2 = u, DF = (r2 - r) cf (AAR) or r - r2 (PGR / PL2R), and the history
// column dx = (u - x) + hb DF.  AAR only ever uses DX_j + beta DF_j
// (AAR.c:228), so it stores that combination (hb = beta); PGR / PL2R store
// DX itself (hb = 0).
template <typename T, int MODE>
struct RichOp {
    static constexpr int NACC = 0;
    static constexpr bool DF = std::is_same<T, double>::value;
    using Raw = Pair<T>;    // (x, r)
    using Ctr = Triple<T>;  // (b, x, r) at the centre
    const T *x;
    const T *r;
    const T *b;
    T *x2;
    T *r2;
    T *dx;
    T *df;
    T c;   // omega * cf
    T cf;  // 1/diag (or 1 without preconditioning)
    T hb;  // beta (AAR) or 0
    double *partials;
    const DevCtrl *ctrl;
    float2 cp, cfp, hbp;  // c, cf, hb as double-float pairs (double-float march)
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {
        if constexpr (DF) {
            cp = df_weight((double)c);
            cfp = df_weight((double)cf);
            hbp = df_weight((double)hb);
        }
    }
    __device__ __forceinline__ Raw fetch(unsigned i) const { return Raw{ldg(x + i), ldg(r + i)}; }
    __device__ __forceinline__ T value(const Raw &v) const { return fma(c, v.b, v.a); }
    // u = x + c r formed in FP64 (as the reference updates x, on the FP64 pipe
    // the double-float sums leave idle) and split once into a float pair
    static constexpr bool VALUE_DF = DF;
    __device__ __forceinline__ float2 value_df(const Raw &v, int k, bool &bad) const {
        return df_split(fma(c, v.b, v.a), k, bad);
    }
    __device__ __forceinline__ Ctr fetch_center(unsigned i) const {
        return Ctr{ldg(b + i), ldg(x + i), ldg(r + i)};
    }
    __device__ __forceinline__ void store(unsigned i, T u, T au, const Ctr &cc, Acc<T> *) const {
        const T rn = cc.a - au;
        const T dfv = (MODE == RICH_AAR) ? (rn - cc.c) * cf : (cc.c - rn);
        x2[i] = u;
        r2[i] = rn;
        dx[i] = fma(hb, dfv, u - cc.b);
        df[i] = dfv;
    }
    // Double-float epilogue: A u rounded to a double once, then the FP64
    // epilogue above with x2 = x + c r in FP64 (the reference's update) -- six
    // FP64 operations on the otherwise idle FP64 pipe in place of ~150
    // double-float instructions; rounding Au first adds 2^-53 |Au| to the
    // sums' own ~2^-48 sum_p |w_p| |u|.
    static constexpr bool STORE_DF = DF;
    __device__ __forceinline__ void store_df(unsigned i, float2, float2 au, const Ctr &cc, int k,
                                             Acc<T> *acc) const {
        store(i, fma(c, cc.c, cc.b), (T)df_to_double(au, k), cc, acc);
    }
};

// Richardson step of the FP32 inner solver in residual-recurrence form:
// f = cf r, r2 = r - omega A f, x += omega f (in place), DF = (r2 - r) cf,
// history column H = omega f + beta DF.  Equal in exact arithmetic to the form above; it stages
// one array (r) instead of two and never reads b, and its rounding is
// relative to |r| rather than to |x|.
template <typename T>
struct RichRecurOp {
    static constexpr int NACC = 0;
    using Raw = T;
    using Ctr = T;  // x at the centre
    const T *r;
    T *x;
    T *r2;
    T *dx;
    T *df;
    T c;    // omega * cf
    T cf;
    T hb;   // beta
    double *partials;
    const DevCtrl *ctrl;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {}
    __device__ __forceinline__ Raw fetch(unsigned i) const { return ldg(r + i); }
    __device__ __forceinline__ T value(const Raw &v) const { return v; }
    __device__ __forceinline__ Ctr fetch_center(unsigned i) const { return x[i]; }
    // H = DX + beta DF with DX = c r taken before it is added to x, so the
    // residual recurrence (r, H, DF) never depends on how x is accumulated:
    // this pass and RichLeanOp below give the same r, H and DF bit for bit.
    __device__ __forceinline__ void store(unsigned i, T rc, T ar, const Ctr &xo, Acc<T> *) const {
        const T rn = fma(-c, ar, rc);
        const T dfv = (rn - rc) * cf;
        x[i] = fma(c, rc, xo);
        r2[i] = rn;
        dx[i] = fma(hb, dfv, c * rc);
        df[i] = dfv;
    }
    // two adjacent points (i even): the paired march
    static constexpr bool PAIRED = true;
    __host__ __device__ const void *pair_ptrs_or() const {
        return (const void *)((uintptr_t)r | (uintptr_t)x | (uintptr_t)r2 | (uintptr_t)dx | (uintptr_t)df);
    }
    __device__ __forceinline__ Two<T> fetch_pair(unsigned i) const { return ld_pair(r + i); }
    __device__ __forceinline__ Two<T> center_pair(unsigned i) const { return ld_pair(x + i); }
    __device__ __forceinline__ void store_pair(unsigned i, Two<T> rc, Two<T> ar, Two<T> xo, Acc<T> *) const {
        const T rna = fma(-c, ar.a, rc.a), rnb = fma(-c, ar.b, rc.b);
        const T dfa = (rna - rc.a) * cf, dfb = (rnb - rc.b) * cf;
        st_pair(x + i, fma(c, rc.a, xo.a), fma(c, rc.b, xo.b));
        st_pair(r2 + i, rna, rnb);
        st_pair(dx + i, fma(hb, dfa, c * rc.a), fma(hb, dfb, c * rc.b));
        st_pair(df + i, dfa, dfb);
    }
};

// The same Richardson step with x left out (reads r, writes r', H, DF: four
// vectors instead of six).  Within an extrapolation cycle the steps sum to
//   sum_j DX_j = sum_j H_j - beta (f - f_start),   f = cf r,
// since the cycle's DF columns telescope; the lean update rebuilds x from the
// cycle-start x and residual and the cycle's H columns (aar_update_block).
template <typename T>
struct RichLeanOp {
    static constexpr int NACC = 0;
    using Raw = T;
    using Ctr = NoCtr;
    const T *r;
    T *r2;
    T *dx;
    T *df;
    T c;    // omega * cf
    T cf;
    T hb;   // beta
    double *partials;
    const DevCtrl *ctrl;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {}
    __device__ __forceinline__ Raw fetch(unsigned i) const { return ldg(r + i); }
    __device__ __forceinline__ T value(const Raw &v) const { return v; }
    __device__ __forceinline__ Ctr fetch_center(unsigned) const { return NoCtr{}; }
    __device__ __forceinline__ void store(unsigned i, T rc, T ar, const Ctr &, Acc<T> *) const {
        const T rn = fma(-c, ar, rc);
        const T dfv = (rn - rc) * cf;
        r2[i] = rn;
        dx[i] = fma(hb, dfv, c * rc);
        df[i] = dfv;
    }
    static constexpr bool PAIRED = true;
    static constexpr bool PACKED = true;
    __host__ __device__ const void *pair_ptrs_or() const {
        return (const void *)((uintptr_t)r | (uintptr_t)r2 | (uintptr_t)dx | (uintptr_t)df);
    }
    __device__ __forceinline__ Two<T> fetch_pair(unsigned i) const { return ld_pair(r + i); }
    __device__ __forceinline__ Two<T> center_pair(unsigned) const { return Two<T>{T(0), T(0)}; }
    __device__ __forceinline__ void store_pair(unsigned i, Two<T> rc, Two<T> ar, Two<T>, Acc<T> *) const {
        const T rna = fma(-c, ar.a, rc.a), rnb = fma(-c, ar.b, rc.b);
        const T dfa = (rna - rc.a) * cf, dfb = (rnb - rc.b) * cf;
        st_pair(r2 + i, rna, rnb);
        st_pair(dx + i, fma(hb, dfa, c * rc.a), fma(hb, dfb, c * rc.b));
        st_pair(df + i, dfa, dfb);
    }
};

// Extrapolation-step residual of the FP32 inner solver: the update kernel
// leaves the step s = x_new - x_old in a scratch vector, so r_new = r - A s
// (r in place), DF_col = (r_new - r) cf, H_col = s + beta DF_col, ||r_new||^2.
template <typename T>
struct ResRecurOp {
    static constexpr int NACC = 1;
    using Raw = T;
    using Ctr = T;  // r at the centre
    const T *dxc;
    T *r;
    T *df;
    T *hc;
    T cf;
    T hb;
    double *partials;
    const DevCtrl *ctrl;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {}
    __device__ __forceinline__ Raw fetch(unsigned i) const { return ldg(dxc + i); }
    __device__ __forceinline__ T value(const Raw &v) const { return v; }
    __device__ __forceinline__ Ctr fetch_center(unsigned i) const { return r[i]; }
    __device__ __forceinline__ void store(unsigned i, T step, T au, const Ctr &ro, Acc<T> *acc) const {
        const T rn = ro - au;
        const T dfv = (rn - ro) * cf;
        df[i] = dfv;
        hc[i] = fma(hb, dfv, step);
        r[i] = rn;
        acc[0].add_prod(rn, rn);
    }
    // two adjacent points (i even): the paired march
    static constexpr bool PAIRED = true;
    __host__ __device__ const void *pair_ptrs_or() const {
        return (const void *)((uintptr_t)dxc | (uintptr_t)r | (uintptr_t)df | (uintptr_t)hc);
    }
    __device__ __forceinline__ Two<T> fetch_pair(unsigned i) const { return ld_pair(dxc + i); }
    __device__ __forceinline__ Two<T> center_pair(unsigned i) const { return ld_pair(r + i); }
    __device__ __forceinline__ void store_pair(unsigned i, Two<T> st, Two<T> au, Two<T> ro, Acc<T> *acc) const {
        const T rna = ro.a - au.a, rnb = ro.b - au.b;
        const T dfa = (rna - ro.a) * cf, dfb = (rnb - ro.b) * cf;
        st_pair(df + i, dfa, dfb);
        st_pair(hc + i, fma(hb, dfa, st.a), fma(hb, dfb, st.b));
        st_pair(r + i, rna, rnb);
        acc[0].add_prod(rna, rna);
        acc[0].add_prod(rnb, rnb);
    }
};

// CG: d_new = cf r + beta d_old at every stencil point, q = A d_new, d.q.
template <typename T>
struct CgDirOp {
    static constexpr int NACC = 1;
    static constexpr bool DF = std::is_same<T, double>::value;
    using Raw = Pair<T>;  // (r, d_old)
    using Ctr = NoCtr;
    const T *r;
    const T *d_old;
    T *d_new;
    T *q;
    T cf;
    T beta;
    double *partials;
    const DevCtrl *ctrl;
    float2 cfp, betap;  // cf, beta as double-float pairs (double-float march)
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {
        beta = (T)ctrl->beta;
        if constexpr (DF) {
            cfp = df_weight((double)cf);
            betap = df_weight((double)beta);
        }
    }
    __device__ __forceinline__ Raw fetch(unsigned i) const { return Raw{ldg(r + i), ldg(d_old + i)}; }
    __device__ __forceinline__ T value(const Raw &v) const { return fma(beta, v.b, cf * v.a); }
    // d = cf r + beta d_old formed in FP64 (on the FP64 pipe the double-float
    // sums leave idle) and split once into the pair the sums use; the stored
    // direction is that pair, rounded once
    static constexpr bool VALUE_DF = DF;
    __device__ __forceinline__ float2 value_df(const Raw &v, int k, bool &bad) const {
        return df_split(value(v), k, bad);
    }
    __device__ __forceinline__ Ctr fetch_center(unsigned) const { return Ctr{}; }
    __device__ __forceinline__ void store(unsigned i, T u, T au, const Ctr &, Acc<T> *acc) const {
        d_new[i] = u;
        q[i] = au;
        acc[0].add_prod(u, au);
    }
};

// FP64 refinement residual: r32 = float(b - A x), ||b - A x||^2 in FP64
// (T64 / T32: double / float or their complex forms).
template <typename T64, typename T32>
struct IrResidualOp {
    static constexpr int NACC = 1;
    static constexpr bool DF = IsDfMarch<T64>::value;  // FP64 and complex128
    using Raw = T64;
    using Ctr = T64;  // b
    const T64 *x;
    const T64 *b;
    T32 *r32;
    double *partials;
    const DevCtrl *ctrl;
    int zgate;  // 1: stand down when ctrl->x_zero (ir_residual_const serves)
    __device__ bool skip() const { return solve_done(ctrl) || (zgate && ctrl->x_zero); }
    __device__ void init() {}
    __device__ __forceinline__ Raw fetch(unsigned i) const { return ldg(x + i); }
    __device__ __forceinline__ T64 value(const Raw &v) const { return v; }
    __device__ __forceinline__ Ctr fetch_center(unsigned i) const { return ldg(b + i); }
    __device__ __forceinline__ void store(unsigned i, T64, T64 au, const Ctr &bb, Acc<T64> *acc) const {
        const T64 rn = bb - au;
        r32[i] = (T32)rn;
        acc[0].add_prod(rn, rn);
    }
    // A u rounded to a double (each part) once, then the FP64 epilogue of store().
    static constexpr bool STORE_DF = DF;
    template <class V>
    __device__ __forceinline__ void store_df(unsigned i, V, V au, const Ctr &bb, int k, Acc<T64> *acc) const {
        if constexpr (DF) store(i, T64(0), DfMarch<T64>::to_double(au, k), bb, acc);
    }
};

// Richardson step of the residual ring: r2 = r - c A r and nothing else (two
// vectors per pass); the column's DF and H are rebuilt from r and r2 where
// they are read (RingWindow).  r2 is RichLeanOp's r2 bit for bit.
template <typename T>
struct RichRingOp {
    static constexpr int NACC = 0;
    using Raw = T;
    using Ctr = NoCtr;
    const T *r;
    T *r2;
    T c;  // omega * cf
    double *partials;
    const DevCtrl *ctrl;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {}
    __device__ __forceinline__ Raw fetch(unsigned i) const { return ldg(r + i); }
    __device__ __forceinline__ T value(const Raw &v) const { return v; }
    __device__ __forceinline__ Ctr fetch_center(unsigned) const { return NoCtr{}; }
    __device__ __forceinline__ void store(unsigned i, T rc, T ar, const Ctr &, Acc<T> *) const {
        r2[i] = fma(-c, ar, rc);
    }
    static constexpr bool PAIRED = true;
    static constexpr bool PACKED = false;  // packed sums spill here and ran 5% slower
    __host__ __device__ const void *pair_ptrs_or() const { return (const void *)((uintptr_t)r | (uintptr_t)r2); }
    __device__ __forceinline__ Two<T> fetch_pair(unsigned i) const { return ld_pair(r + i); }
    __device__ __forceinline__ Two<T> center_pair(unsigned) const { return Two<T>{T(0), T(0)}; }
    __device__ __forceinline__ void store_pair(unsigned i, Two<T> rc, Two<T> ar, Two<T>, Acc<T> *) const {
        st_pair(r2 + i, fma(-c, ar.a, rc.a), fma(-c, ar.b, rc.b));
    }
};

// Extrapolation-step residual of the residual ring: r2 = r - A step into the
// next ring slot (r stays), H_col = step + beta DF_col stored, ||r2||^2; DF_col
// is rebuilt from r and r2.  The arithmetic of ResRecurOp.
template <typename T>
struct ResRingOp {
    static constexpr int NACC = 1;
    using Raw = T;
    using Ctr = T;  // r at the centre
    const T *stp;
    const T *r;
    T *r2;
    T *hc;
    T cf;
    T hb;
    double *partials;
    const DevCtrl *ctrl;
    __device__ bool skip() const { return solve_done(ctrl); }
    __device__ void init() {}
    __device__ __forceinline__ Raw fetch(unsigned i) const { return ldg(stp + i); }
    __device__ __forceinline__ T value(const Raw &v) const { return v; }
    __device__ __forceinline__ Ctr fetch_center(unsigned i) const { return ldg(r + i); }
    __device__ __forceinline__ void store(unsigned i, T step, T au, const Ctr &ro, Acc<T> *acc) const {
        const T rn = ro - au;
        const T dfv = (rn - ro) * cf;
        hc[i] = fma(hb, dfv, step);
        r2[i] = rn;
        acc[0].add_prod(rn, rn);
    }
    static constexpr bool PAIRED = true;
    __host__ __device__ const void *pair_ptrs_or() const {
        return (const void *)((uintptr_t)stp | (uintptr_t)r | (uintptr_t)r2 | (uintptr_t)hc);
    }
    __device__ __forceinline__ Two<T> fetch_pair(unsigned i) const { return ld_pair(stp + i); }
    __device__ __forceinline__ Two<T> center_pair(unsigned i) const { return ld_pair(r + i); }
    __device__ __forceinline__ void store_pair(unsigned i, Two<T> st, Two<T> au, Two<T> ro, Acc<T> *acc) const {
        const T rna = ro.a - au.a, rnb = ro.b - au.b;
        const T dfa = (rna - ro.a) * cf, dfb = (rnb - ro.b) * cf;
        st_pair(hc + i, fma(hb, dfa, st.a), fma(hb, dfb, st.b));
        st_pair(r2 + i, rna, rnb);
        acc[0].add_prod(rna, rna);
        acc[0].add_prod(rnb, rnb);
    }
};

// ---------------------------------------------------------------- stencil dispatch

template <class Op, class = void> struct IsPaired { static constexpr bool value = false; };
template <class Op> struct IsPaired<Op, std::void_t<decltype(Op::PAIRED)>> { static constexpr bool value = Op::PAIRED; };


template <typename T, class Op>
inline bool paired_ok(const StencilLaunch &L, const Weights<T> &w, const Op &op) {
    if constexpr (IsPaired<Op>::value && std::is_same<T, float>::value) {
        return w.radius == 6 && L.tile == 0 && (L.g.nx % 2) == 0 && (((uintptr_t)op.pair_ptrs_or()) & 7u) == 0;
    } else {
        return false;
    }
}

// z depth and block count of the paired march on grid g (64-wide tiles, the
// paired kernel's residency); 0 blocks when T has no paired march.
template <typename T>
long long Kernels<T>::paired_plan(const Geom &g, int *lz) {
    if constexpr (std::is_same<T, float>::value) {
        static int slots = 0;
        if (slots == 0) {
            int occ = 0, dev = 0, sms = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &occ, stencil_x2_kernel<T, kPairBY, kPairNY, kPairMINB, RichLeanOp<T>>, 32 * kPairBY, 0) !=
                    cudaSuccess ||
                occ < 1) {
                cudaGetLastError();
                occ = 1;
            }
            slots = std::max(1, sms) * occ;
        }
        const int z = balanced_lz(g, kPairBY * kPairNY, slots, FillCost<T>::value, 64);
        if (lz) *lz = z;
        return (long long)((g.nx + 63) / 64) * ((g.ny + kPairBY * kPairNY - 1) / (kPairBY * kPairNY)) *
               ((g.nz + z - 1) / z);
    } else {
        (void)g;
        if (lz) *lz = 0;
        return 0;
    }
}

template <typename T>
int Kernels<T>::paired_blocks_per_sm(int shape) {
    if constexpr (std::is_same<T, float>::value) {
        int occ = 0;
        const cudaError_t e =
            shape == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                             &occ, stencil_x2_kernel<T, kPair3BY, kPair3NY, kPair3MINB, RichRingOp<T>>, 32 * kPair3BY, 0)
            : shape == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                             &occ, stencil_x2_kernel<T, kPair2BY, kPair2NY, kPair2MINB, RichLeanOp<T>>, 32 * kPair2BY, 0)
                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                             &occ, stencil_x2_kernel<T, kPairBY, kPairNY, kPairMINB, RichLeanOp<T>>, 32 * kPairBY, 0);
        if (e != cudaSuccess || occ < 1) {
            cudaGetLastError();
            occ = 1;
        }
        return occ;
    } else {
        (void)shape;
        return 0;
    }
}

template <typename T, int BY, int NY, int MB, class Op>
cudaError_t launch_x2(const StencilLaunch &L, const Weights<T> &w, const Op &op) {
    const dim3 grid((unsigned)((L.g.nx + 63) / 64), (unsigned)((L.g.ny + BY * NY - 1) / (BY * NY)),
                    (unsigned)((L.g.nz + L.lz - 1) / L.lz));
    stencil_x2_kernel<T, BY, NY, MB, Op><<<grid, dim3(32, BY), 0, L.stream>>>(L.g, w, L.lz, op);
    return cudaGetLastError();
}

template <typename T, int V, class Op>
cudaError_t launch_stencil_var(const StencilLaunch &L, const Weights<T> &w, const Op &op) {
    constexpr int BY = TileVar<T, V>::BY, NY = TileVar<T, V>::NY, MB = TileVar<T, V>::MINB;
    const dim3 grid = stencil_grid(L.g, BY * NY, L.lz);
    if constexpr (DfOk<Op>::value) {
        if (!L.exact) {
            stencil_kernel<T, 6, BY, NY, MB, false, Op, true><<<grid, dim3(32, BY), 0, L.stream>>>(L.g, w, L.lz, op);
            return cudaGetLastError();
        }
    }
    stencil_kernel<T, 6, BY, NY, MB, false, Op><<<grid, dim3(32, BY), 0, L.stream>>>(L.g, w, L.lz, op);
    return cudaGetLastError();
}

// Passes that write partial sums keep the default tile (their block count
// sizes the partials); the others may run any tuned variant.
template <typename T, class Op>
cudaError_t launch_stencil(const StencilLaunch &L, const Weights<T> &w, const Op &op) {
    constexpr int BY = TileOf<T>::BY, NY = TileOf<T>::NY;
    // L.paired: the caller planned this launch as the paired march (its z depth
    // in L.lz, its block count in the caller's partial-sum bookkeeping)
    if (L.paired >= 1) {
        if constexpr (IsPaired<Op>::value && std::is_same<T, float>::value) {
            if (!paired_ok<T>(L, w, op)) return cudaErrorInvalidValue;
            if (L.paired == 1) return launch_x2<T, kPairBY, kPairNY, kPairMINB>(L, w, op);
            if constexpr (Op::NACC == 0) {
                if (L.paired == 2) return launch_x2<T, kPair2BY, kPair2NY, kPair2MINB>(L, w, op);
                if (L.paired == 3) return launch_x2<T, kPair3BY, kPair3NY, kPair3MINB>(L, w, op);
            }
            return cudaErrorInvalidValue;
        } else {
            return cudaErrorInvalidValue;
        }
    }
    if (w.radius == 6) {
        if constexpr (Op::NACC == 0) {
            if (L.tile == 1) return launch_stencil_var<T, 1>(L, w, op);
            if (L.tile == 2) return launch_stencil_var<T, 2>(L, w, op);
        }
        return launch_stencil_var<T, 0>(L, w, op);
    }
    const dim3 grid = stencil_grid(L.g, BY * NY, L.lz);
    if constexpr (DfOk<Op>::value) {
        if (!L.exact) {
            stencil_kernel<T, LSG_MAX_RADIUS, BY, NY, 1, true, Op, true>
                <<<grid, dim3(32, BY), 0, L.stream>>>(L.g, w, L.lz, op);
            return cudaGetLastError();
        }
    }
    stencil_kernel<T, LSG_MAX_RADIUS, BY, NY, 1, true, Op><<<grid, dim3(32, BY), 0, L.stream>>>(L.g, w, L.lz, op);
    return cudaGetLastError();
}

// Resident blocks per SM of the Richardson pass in tile variant V.
template <typename T, int V>
static int rich_blocks_per_sm() {
    using Tl = TileVar<T, V>;
    using Op = typename std::conditional<std::is_same<typename RealOf<T>::type, float>::value, RichLeanOp<T>,
                                         RichOp<T, RICH_AAR>>::type;
    int n = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &n, stencil_kernel<T, 6, Tl::BY, Tl::NY, Tl::MINB, false, Op, DfOk<Op>::value>, 32 * Tl::BY, 0);
    if (e != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    return n;
}

template <typename T>
int Kernels<T>::stencil_blocks_per_sm(int var) {
    if (var == 1) return rich_blocks_per_sm<T, 1>();
    if (var == 2) return rich_blocks_per_sm<T, 2>();
    return rich_blocks_per_sm<T, 0>();
}

// ---------------------------------------------------------------- point-local kernels

// Gram partials for history depth M (register accumulators), VEC consecutive
// points per thread and step (one 16-byte load per vector).  FP32 vectors:
// the VEC products of a step are summed in FP32 and folded into a
// double-float accumulator (lsg_accum.cuh); FP64 vectors: FP64 FMAs.
// True when every pointer is 16-byte aligned (nullptr counts as aligned).
template <typename... P>
__host__ __device__ inline bool aligned16(const P *...p) {
    return ((((uintptr_t)p) | ... | (uintptr_t)0) & 15u) == 0;
}

template <typename T> struct Vec4;
template <> struct Vec4<float> { using type = float4; static constexpr int N = 4; };
template <> struct Vec4<double> { using type = double2; static constexpr int N = 2; };

template <typename V> __device__ __forceinline__ V ldv(const V *p) { return ldg(p); }

__device__ __forceinline__ float dotv(const float4 &a, const float4 &b) {
    float p = a.x * b.x;
    p = fmaf(a.y, b.y, p);
    p = fmaf(a.z, b.z, p);
    return fmaf(a.w, b.w, p);
}
__device__ __forceinline__ void accv(Acc<float> &acc, const float4 &a, const float4 &b) { acc.add(dotv(a, b)); }
__device__ __forceinline__ void accv(Acc<double> &acc, const double2 &a, const double2 &b) {
    acc.add_prod(a.x, b.x);
    acc.add_prod(a.y, b.y);
}

__device__ __forceinline__ void accv(Acc<float> &acc, float a, float b) { acc.add_prod(a, b); }
__device__ __forceinline__ void accv(Acc<double> &acc, double a, double b) { acc.add_prod(a, b); }

// Loads of VN consecutive values (VEC) or of one value.
template <typename T, bool VEC> struct VecLoad { using type = T; static constexpr int N = 1; };
template <typename T> struct VecLoad<T, true> { using type = typename Vec4<T>::type; static constexpr int N = Vec4<T>::N; };

// One block's share of the Gram sums: block `blk` of `nblk` covering points
// 0..n-1 of the history (grid-stride), NV sums written to out[0..NV).
template <typename T, int KIND, int M, bool VEC>
__device__ __forceinline__ void gram_block(const T *__restrict__ dx, const T *__restrict__ df,
                                           const T *__restrict__ r, long long n, double *out,
                                           long long blk, long long nblk) {
    using V = typename VecLoad<T, VEC>::type;
    constexpr int VN = VecLoad<T, VEC>::N;
    constexpr int NP = (KIND == GRAM_SYM) ? (M * (M + 1)) / 2 : M * M;
    constexpr int NV = NP + M;
    __shared__ double red[NV * (kReduceThreads / 32)];
    Acc<T> acc[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) acc[k].zero();
    const long long nv = n / VN;  // VEC: caller guarantees n % VN == 0
    const V *dfv = reinterpret_cast<const V *>(df);
    const V *dxv = reinterpret_cast<const V *>(dx);
    const V *rvv = reinterpret_cast<const V *>(r);
    const long long stride = nblk * blockDim.x;
    for (long long i = blk * blockDim.x + threadIdx.x; i < nv; i += stride) {
        V f[M], xv[KIND == GRAM_SYM ? 1 : M];
#pragma unroll
        for (int j = 0; j < M; j++) f[j] = ldv(dfv + j * nv + i);
        if (KIND == GRAM_GALERKIN) {
#pragma unroll
            for (int j = 0; j < M; j++) xv[j] = ldv(dxv + j * nv + i);
        }
        const V rv = ldv(rvv + i);
        int k = 0;
        if (KIND == GRAM_SYM) {
#pragma unroll
            for (int j = 0; j < M; j++)
#pragma unroll
                for (int a = 0; a <= j; a++) { accv(acc[k], f[a], f[j]); k++; }
#pragma unroll
            for (int j = 0; j < M; j++) accv(acc[NP + j], f[j], rv);
        } else {
#pragma unroll
            for (int a = 0; a < M; a++)
#pragma unroll
                for (int j = 0; j < M; j++) { accv(acc[k], xv[a], f[j]); k++; }
#pragma unroll
            for (int j = 0; j < M; j++) accv(acc[NP + j], xv[j], rv);
        }
    }
    block_reduce_store<NV>(acc, red, out);
}

// The FP64 Gram in double-float arithmetic on the FP32 pipe (the solvers'
// default double-float mode; GB300 runs FP64 at ~1/64 of FP32, which bound
// the FP64 form at ~6x its DRAM time).  Each double is split once into a float
// pair scaled by 2^k (df_split, k from ||b||), each product is formed by the
// FMA two-product with its cross terms (~2^-47 relative, the rounding of a
// thread's FP64 running sum of ~50 products), sums are double-float pairs,
// and the block totals are converted to doubles and scaled back by 2^-2k.
__device__ __forceinline__ void acc_prod_df(Acc<float> &acc, float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    float s, t;
    two_sum(acc.hi, p, s, t);
    acc.hi = s;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(t, e));
}

template <int KIND, int M>
__global__ void __launch_bounds__(kReduceThreads) gram_df_kernel(const double *__restrict__ dx,
                                                                 const double *__restrict__ df,
                                                                 const double *__restrict__ r, long long n,
                                                                 double *partials, DevCtrl *ctrl) {
    constexpr int NP = (KIND == GRAM_SYM) ? (M * (M + 1)) / 2 : M * M;
    constexpr int NV = NP + M;
    __shared__ double red[NV * (kReduceThreads / 32)];
    if (solve_done(ctrl)) return;
    const int k = ctrl ? df_shift_for(ctrl->rhs_norm) : 0;
    bool bad = false;
    Acc<float> acc[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q].zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float2 f[M], xv[KIND == GRAM_SYM ? 1 : M];
#pragma unroll
        for (int j = 0; j < M; j++) f[j] = df_split(ldg(df + j * n + i), k, bad);
        if (KIND == GRAM_GALERKIN) {
#pragma unroll
            for (int j = 0; j < M; j++) xv[j] = df_split(ldg(dx + j * n + i), k, bad);
        }
        const float2 rv = df_split(ldg(r + i), k, bad);
        int q = 0;
        if (KIND == GRAM_SYM) {
#pragma unroll
            for (int j = 0; j < M; j++)
#pragma unroll
                for (int a = 0; a <= j; a++) { acc_prod_df(acc[q], f[a], f[j]); q++; }
#pragma unroll
            for (int j = 0; j < M; j++) acc_prod_df(acc[NP + j], f[j], rv);
        } else {
#pragma unroll
            for (int a = 0; a < M; a++)
#pragma unroll
                for (int j = 0; j < M; j++) { acc_prod_df(acc[q], xv[a], f[j]); q++; }
#pragma unroll
            for (int j = 0; j < M; j++) acc_prod_df(acc[NP + j], xv[j], rv);
        }
    }
    const double us = ldexp(1.0, -k);  // (u 2^k)(v 2^k): scale back by 2^-k twice
    block_reduce_store<NV>(acc, red, partials + (long long)blockIdx.x * NV, nullptr, us, us);
    if (__syncthreads_or(bad ? 1 : 0) && threadIdx.x == 0 && ctrl) atomicOr(&ctrl->df_range, 1);
}

template <typename T, int KIND, int M>
__global__ void __launch_bounds__(kReduceThreads) gram_kernel(const T *__restrict__ dx,
                                                              const T *__restrict__ df,
                                                              const T *__restrict__ r, long long n,
                                                              double *partials,
                                                              const DevCtrl *ctrl) {
    constexpr int NV = ((KIND == GRAM_SYM) ? (M * (M + 1)) / 2 : M * M) + M;
    if (solve_done(ctrl)) return;
    gram_block<T, KIND, M, true>(dx, df, r, n, partials + (long long)blockIdx.x * NV, blockIdx.x, gridDim.x);
}

// ---- Gram by bulk copies (FP32, symmetric kind, m <= 8).  The history
// streams through a ring of kGramStages shared-memory stages; one thread arms
// each stage's mbarrier with the byte count and issues one bulk copy
// (cp.async.bulk) per column, so the loads of the next stages are in flight
// while the block reduces the current one and no warp stalls on a global
// load.  A stage holds one float4 per thread of every column (a 1024-float
// chunk); block b takes chunks b, b + G, ..., so each thread visits the same
// points in the same order as gram_block's grid-stride loop and the sums are
// bit-identical to it.  Every wait is bounded: a copy that has not landed
// after `wait_cycles` SM clocks (a launch parameter: kWaitCycles, ~2 s, in
// solves) sets LSG_TIMEOUT in the control block, the block waits (again
// bounded) for its own copies in flight and returns.
constexpr int kGramStages = 3;
constexpr int kGramChunk = 4 * kReduceThreads;  // floats per column per stage
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz: the solves' limit

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(b))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *b, unsigned phase) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(phase)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *b, unsigned phase, long long limit) {
    if (mbar_try_wait(b, phase)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(b, phase))
        if (clock64() - t0 > limit) return false;
    return true;
}

// extra_tx: bytes armed on each stage beyond the copies' (0; the failure
// test arms more, so the waits run out and the timeout path is taken);
// wait_cycles: the limit of every wait.
// RING: the columns come from the residual ring (RingWindow rw, slots ss
// floats apart): the stage holds r_{it-m-1} .. r_{it-1} in time order, the
// block rebuilds DF_t = (r_t+1 - r_t) cf (stored columns, rw.dfmem, straight
// from df), accumulates in time order and writes each sum at its column-order
// place, so the partials equal gram()'s over the same columns bit for bit.
// FULL (RING): every column valid and none stored (rw.valid all ones,
// rw.dfmem 0, the steady state): the per-column tests, which cost ~10% of
// the pass at 256^3, are compiled out.
template <int M, bool RING = false, bool FULL = false>
__global__ void __launch_bounds__(kReduceThreads, 2) gram_bulk_kernel(const float *__restrict__ df,
                                                                     const float *__restrict__ r, long long n,
                                                                     double *partials, DevCtrl *ctrl,
                                                                     unsigned extra_tx, long long wait_cycles,
                                                                     const float *__restrict__ ring = nullptr,
                                                                     long long ss = 0, RingWindow rw = {},
                                                                     float cf = 1.f) {
    constexpr int NP = (M * (M + 1)) / 2;
    constexpr int NV = NP + M;
    constexpr int S = kGramStages, CH = kGramChunk, CV = CH / 4;
    extern __shared__ __align__(128) float gsm[];  // S stages x (M + 1) columns x CH floats
    __shared__ __align__(8) unsigned long long full[S];
    __shared__ double red[NV * (kReduceThreads / 32)];
    __shared__ int abort_flag;
    __shared__ int perm[RING ? NV : 1];
    if (solve_done(ctrl)) return;
    const int tid = threadIdx.x;
    const long long nchunk = (n + CH - 1) / CH;
    const long long first = blockIdx.x, step = gridDim.x;
    const long long mine = first < nchunk ? (nchunk - 1 - first) / step + 1 : 0;
    if (tid == 0) {
        for (int st = 0; st < S; st++) mbar_init(&full[st], 1);
        abort_flag = 0;
        mbar_init_fence();
    }
    if constexpr (RING) {
        if (tid < NV) {  // time-order sum -> column-order place
            int o;
            if (tid < NP) {
                int tj = 0;
                while ((tj + 1) * (tj + 2) / 2 <= tid) tj++;
                const int ta = tid - tj * (tj + 1) / 2;
                const int ca = (rw.s0 + ta) % M, cj = (rw.s0 + tj) % M;
                const int lo = ca < cj ? ca : cj, hi = ca < cj ? cj : ca;
                o = hi * (hi + 1) / 2 + lo;
            } else {
                o = NP + (rw.s0 + tid - NP) % M;
            }
            perm[tid] = o;
        }
    }
    __syncthreads();
    auto issue = [&](long long k) {  // the block's k-th chunk into stage k % S (thread 0)
        const long long off = (first + k * step) * CH;
        const unsigned bytes = (unsigned)(min((long long)CH, n - off) * 4);
        unsigned long long *bar = &full[k % S];
        float *dst = gsm + (size_t)(k % S) * (M + 1) * CH;
        mbar_expect_tx(bar, bytes * (M + 1) + extra_tx);
        if constexpr (RING) {
#pragma unroll
            for (int v = 0; v <= M; v++) bulk_g2s(dst + v * CH, ring + (long long)rw.slot[v] * ss + off, bytes, bar);
        } else {
#pragma unroll
            for (int v = 0; v < M; v++) bulk_g2s(dst + v * CH, df + (long long)v * n + off, bytes, bar);
            bulk_g2s(dst + M * CH, r + off, bytes, bar);
        }
    };
    if (tid == 0)
        for (long long k = 0; k < S && k < mine; k++) issue(k);
    Acc<float> acc[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) acc[k].zero();
    long long k = 0;
    for (; k < mine; k++) {
        const int st = (int)(k % S);
        if (!mbar_wait_bounded(&full[st], (unsigned)((k / S) & 1), wait_cycles)) {
            abort_flag = 1;
        } else {
            const long long off = (first + k * step) * CH;
            if (off + 4 * tid < n) {
                const float4 *src = reinterpret_cast<const float4 *>(gsm + (size_t)st * (M + 1) * CH);
                float4 f[M];
                float4 rv;
                if constexpr (RING) {
                    float4 u[M + 1];
#pragma unroll
                    for (int v = 0; v <= M; v++) u[v] = src[v * CV + tid];
#pragma unroll
                    for (int t = 0; t < M; t++) {
                        float4 d;
                        if (!FULL && ((rw.dfmem >> t) & 1u)) {
                            d = ldg(reinterpret_cast<const float4 *>(df + (long long)((rw.s0 + t) % M) * n + off) + tid);
                        } else {
                            d.x = (u[t + 1].x - u[t].x) * cf;
                            d.y = (u[t + 1].y - u[t].y) * cf;
                            d.z = (u[t + 1].z - u[t].z) * cf;
                            d.w = (u[t + 1].w - u[t].w) * cf;
                        }
                        if (!FULL && !((rw.valid >> t) & 1u)) d = make_float4(0.f, 0.f, 0.f, 0.f);
                        f[t] = d;
                    }
                    rv = u[M];
                } else {
#pragma unroll
                    for (int v = 0; v < M; v++) f[v] = src[v * CV + tid];
                    rv = src[M * CV + tid];
                }
                int q = 0;
#pragma unroll
                for (int j = 0; j < M; j++)
#pragma unroll
                    for (int a = 0; a <= j; a++) { accv(acc[q], f[a], f[j]); q++; }
#pragma unroll
                for (int j = 0; j < M; j++) accv(acc[NP + j], f[j], rv);
            }
        }
        __syncthreads();  // stage st is free again (and abort_flag is seen by all)
        if (abort_flag) break;
        if (tid == 0 && k + S < mine) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(k + S);
        }
    }
    if (abort_flag) {
        if (tid == 0) {
            for (long long kk = k; kk < k + S && kk < mine; kk++)
                mbar_wait_bounded(&full[kk % S], (unsigned)((kk / S) & 1), wait_cycles);
            if (ctrl) {
                ctrl->status = LSG_TIMEOUT;
                ctrl->done = 1;
            }
        }
        return;
    }
    block_reduce_store<NV>(acc, red, partials + (long long)blockIdx.x * NV, RING ? perm : nullptr);
}

// LSG_FAULT_GRAM_TX=<bytes>: failure test of the bulk-copy Gram's bounded
// waits (every stage armed with that many bytes more than its copies bring),
// which then give up after LSG_GRAM_WAIT_CYCLES SM clocks (default kWaitCycles).
static inline unsigned gram_fault_tx() {
    static const unsigned v = [] {
        const char *e = getenv("LSG_FAULT_GRAM_TX");
        const long t = e ? atol(e) : 0;
        return (unsigned)(t > 0 && t < 65536 ? t : 0);
    }();
    return v;
}
static inline long long gram_wait_cycles() {
    static const long long v = [] {
        const char *e = getenv("LSG_GRAM_WAIT_CYCLES");
        const long long t = e ? atoll(e) : 0;
        return t >= 1000000 && t <= kWaitCycles ? t : kWaitCycles;
    }();
    return v;
}

template <int M>
static size_t gram_bulk_smem() {
    return (size_t)kGramStages * (M + 1) * kGramChunk * sizeof(float);
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
    __shared__ double red[(kReduceThreads / 32) * AccWidth<T>::value];
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
    __shared__ double out;
    Acc<T> a1[1] = {acc};
    block_reduce_store<1>(a1, red, &out);
    __syncthreads();
    if (threadIdx.x == 0) partials[(long long)blockIdx.x * nv + v] = out;
}

// x_new = x + beta cf r - sum_j H_j s_j with H_j = DX_j + beta DF_j
// (AAR.c:116-117, 225-231); the step x_new - x_old goes to `step`.
// M: history depth known at compile time (all m loads in flight at once),
// VN points per thread and step through 16-byte vectors; M = 0 is the
// generic path (runtime m, scalar).
//   FP64 / complex128 (the reference form): x_new = (x + beta cf r) - am,
//   step = x_new - x, am = sum_j H_j s_j.
//   FP32 residual recurrence: step = beta cf r - am first, x_new = x + step,
//   so the step (the next residual's stencil input) does not depend on x.
//   LEAN (FP32 with x left out of the Richardson passes): x holds the
//   cycle-start iterate, rs the cycle-start residual, and bit j of `mask`
//   marks the H columns the cycle's Richardson passes wrote;
//   x_new = x + (sum_mask H_j - beta cf (r - rs)) + step.
template <typename T, bool LEAN>
__device__ __forceinline__ void update_point(T xo, T ro, T rso, T am, T ac, T beta, T cf, T &xn, T &st) {
    if constexpr (!std::is_same<typename RealOf<T>::type, float>::value) {
        xn = fma(beta, ro * cf, xo) - am;
        st = xn - xo;
    } else if constexpr (!LEAN) {
        st = beta * (ro * cf) - am;
        xn = xo + st;
    } else {
        st = beta * (ro * cf) - am;
        xn = xo + ((ac - beta * ((ro - rso) * cf)) + st);
    }
}

template <typename T, int M, bool VEC, bool LEAN = false>
__device__ __forceinline__ void aar_update_block(int m, T *__restrict__ x, const T *__restrict__ r,
                                                 const T *__restrict__ h, T *__restrict__ step,
                                                 T beta, T cf, long long n, const DevCtrl *ctrl,
                                                 long long blk, long long nblk,
                                                 const T *__restrict__ rs = nullptr, unsigned mask = 0u) {
    __shared__ T s[LSG_MAX_M];
    if (threadIdx.x < m) s[threadIdx.x] = ctrl_s<T>(ctrl, threadIdx.x);
    __syncthreads();
    const long long stride = nblk * blockDim.x;
    const long long t0 = blk * blockDim.x + threadIdx.x;
    if constexpr (M > 0) {
        using V = typename VecLoad<T, VEC>::type;
        constexpr int VN = VecLoad<T, VEC>::N;
        const long long nv = n / VN;  // VEC: caller guarantees n % VN == 0
        const V *hv = reinterpret_cast<const V *>(h);
        V *xv = reinterpret_cast<V *>(x);
        const V *rv = reinterpret_cast<const V *>(r);
        const V *rsv = reinterpret_cast<const V *>(rs);
        V *sv = reinterpret_cast<V *>(step);
        T sj[M], ij[M];
#pragma unroll
        for (int j = 0; j < M; j++) {
            sj[j] = s[j];
            ij[j] = ((mask >> j) & 1u) ? T(1) : T(0);
        }
        for (long long i = t0; i < nv; i += stride) {
            V hj[M];
#pragma unroll
            for (int j = 0; j < M; j++) hj[j] = ldv(hv + j * nv + i);
            const V xo = xv[i], ro = rv[i];
            V rso = ro;
            if constexpr (LEAN) rso = rsv[i];
            const T *xs = (const T *)&xo;
            const T *rr = (const T *)&ro;
            const T *rss = (const T *)&rso;
            V xn, st;
            T *xns = (T *)&xn, *sts = (T *)&st;
#pragma unroll
            for (int e = 0; e < VN; e++) {
                T am = T(0), ac = T(0);
#pragma unroll
                for (int j = 0; j < M; j++) {
                    am = fma(((const T *)&hj[j])[e], sj[j], am);
                    if constexpr (LEAN) ac = fma(((const T *)&hj[j])[e], ij[j], ac);
                }
                update_point<T, LEAN>(xs[e], rr[e], rss[e], am, ac, beta, cf, xns[e], sts[e]);
            }
            xv[i] = xn;
            sv[i] = st;
        }
    } else {
        for (long long i = t0; i < n; i += stride) {
            T am = T(0), ac = T(0);
            for (int j = 0; j < m; j++) {
                const T hv = ldg(h + j * n + i);
                am = fma(hv, s[j], am);
                if constexpr (LEAN) ac = fma(hv, ((mask >> j) & 1u) ? T(1) : T(0), ac);
            }
            const T ro = r[i];
            T rso = ro;
            if constexpr (LEAN) rso = rs[i];
            T xn, st;
            update_point<T, LEAN>(x[i], ro, rso, am, ac, beta, cf, xn, st);
            x[i] = xn;
            step[i] = st;
        }
    }
}

// One launch of aar_update_block over the whole vector (M, LEAN as there).
template <typename T, int M>
__global__ void __launch_bounds__(kReduceThreads) aar_update_kernel(int m, T *__restrict__ x,
                                                                    const T *__restrict__ r,
                                                                    const T *__restrict__ h,
                                                                    T *__restrict__ step, T beta,
                                                                    T cf, long long n,
                                                                    const DevCtrl *ctrl) {
    if (solve_done(ctrl)) return;
    aar_update_block<T, M, (M > 0)>(m, x, r, h, step, beta, cf, n, ctrl, blockIdx.x, gridDim.x);
}

template <typename T, int M>
__global__ void __launch_bounds__(kReduceThreads) aar_update_lean_kernel(int m, T *__restrict__ x,
                                                                         const T *__restrict__ r,
                                                                         const T *__restrict__ rs,
                                                                         const T *__restrict__ h,
                                                                         T *__restrict__ step, T beta,
                                                                         T cf, long long n, unsigned mask,
                                                                         const DevCtrl *ctrl) {
    if (solve_done(ctrl)) return;
    aar_update_block<T, M, (M > 0), true>(m, x, r, h, step, beta, cf, n, ctrl, blockIdx.x, gridDim.x, rs, mask);
}

// ---- residual-ring extrapolation (FP32, RingWindow).  Per point: the m + 1
// ring residuals r_{it-m-1} .. r_{it-1}, the stored H columns (rw.hmem) and x;
// the other columns' H_t = c r_t + beta (r_t+1 - r_t) cf as the Richardson
// pass rounds it; am = sum_j H_j s_j summed in column order j = 0..m-1 (the
// window's time order rotated by s0, a template parameter), so the step equals
// aar_update's over the same columns bit for bit; x first takes the cycle's
// Richardson steps x = fma(c, r_{k-1}, x) in iteration order, as the
// x-carrying pass applies them.
template <int M, int ROT>
__device__ __forceinline__ void ring_update_loop(const float *__restrict__ ring, long long ss, const RingWindow &rw,
                                                 const float *__restrict__ hm, float *__restrict__ x,
                                                 float *__restrict__ step, float c, float beta, float cf,
                                                 long long n, const float *sj) {
    // one float4 per thread (no grid-stride loop: nothing loop-invariant to keep in registers)
    const long long nv = n / 4;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 *r4 = reinterpret_cast<const float4 *>(ring);
    const long long ss4 = ss / 4;
    const float4 *h4 = reinterpret_cast<const float4 *>(hm);
    float4 *x4 = reinterpret_cast<float4 *>(x);
    float4 *s4 = reinterpret_cast<float4 *>(step);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    {
        float4 u[M + 1];
#pragma unroll
        for (int t = 0; t <= M; t++) u[t] = ldg(r4 + rw.slot[t] * ss4 + i);
        // the first two stored H columns are loaded with the ring (more only when p is small)
        const float4 hx0 = rw.e0 >= 0 ? ldg(h4 + (long long)((ROT + rw.e0) % M) * nv + i) : zero;
        const float4 hx1 = rw.e1 >= 0 ? ldg(h4 + (long long)((ROT + rw.e1) % M) * nv + i) : zero;
        float4 xo = x4[i];
#pragma unroll
        for (int t = 0; t < M; t++)
            if ((rw.cyc >> t) & 1u) {
                xo.x = fma(c, u[t].x, xo.x);
                xo.y = fma(c, u[t].y, xo.y);
                xo.z = fma(c, u[t].z, xo.z);
                xo.w = fma(c, u[t].w, xo.w);
            }
        float4 am = zero;
#pragma unroll
        for (int j = 0; j < M; j++) {
            const int t = (j + M - ROT) % M;  // the column's time in the window
            float4 h;
            if (t == rw.e0) {
                h = hx0;
            } else if (t == rw.e1) {
                h = hx1;
            } else if ((rw.hmem >> t) & 1u) {
                h = ldg(h4 + (long long)j * nv + i);
            } else {
                h.x = fma(beta, (u[t + 1].x - u[t].x) * cf, c * u[t].x);
                h.y = fma(beta, (u[t + 1].y - u[t].y) * cf, c * u[t].y);
                h.z = fma(beta, (u[t + 1].z - u[t].z) * cf, c * u[t].z);
                h.w = fma(beta, (u[t + 1].w - u[t].w) * cf, c * u[t].w);
            }
            if (!((rw.valid >> t) & 1u)) h = zero;
            am.x = fma(h.x, sj[j], am.x);
            am.y = fma(h.y, sj[j], am.y);
            am.z = fma(h.z, sj[j], am.z);
            am.w = fma(h.w, sj[j], am.w);
        }
        float4 xn, st;
        update_point<float, false>(xo.x, u[M].x, u[M].x, am.x, 0.f, beta, cf, xn.x, st.x);
        update_point<float, false>(xo.y, u[M].y, u[M].y, am.y, 0.f, beta, cf, xn.y, st.y);
        update_point<float, false>(xo.z, u[M].z, u[M].z, am.z, 0.f, beta, cf, xn.z, st.z);
        update_point<float, false>(xo.w, u[M].w, u[M].w, am.w, 0.f, beta, cf, xn.w, st.w);
        x4[i] = xn;
        s4[i] = st;
    }
}

template <int M>
__global__ void __launch_bounds__(kReduceThreads) aar_update_ring_kernel(const float *__restrict__ ring, long long ss,
                                                                         RingWindow rw, const float *__restrict__ hm,
                                                                         float *__restrict__ x,
                                                                         float *__restrict__ step, float c,
                                                                         float beta, float cf, long long n,
                                                                         const DevCtrl *ctrl) {
    __shared__ float s[M];
    if (solve_done(ctrl)) return;
    if (threadIdx.x < M) s[threadIdx.x] = ctrl_s<float>(ctrl, threadIdx.x);
    __syncthreads();
    float sj[M];
#pragma unroll
    for (int j = 0; j < M; j++) sj[j] = s[j];
    switch (rw.s0) {
#define LSG_RING_ROT(R) \
    case R: if constexpr (R < M) ring_update_loop<M, R>(ring, ss, rw, hm, x, step, c, beta, cf, n, sj); break;
        LSG_RING_ROT(0) LSG_RING_ROT(1) LSG_RING_ROT(2) LSG_RING_ROT(3)
        LSG_RING_ROT(4) LSG_RING_ROT(5) LSG_RING_ROT(6) LSG_RING_ROT(7)
#undef LSG_RING_ROT
    default: break;
    }
}

// x += the cycle's Richardson steps, x = fma(c, r_{k-1}, x) in iteration order.
static __global__ void __launch_bounds__(kReduceThreads) ring_fold_kernel(int m, const float *__restrict__ ring,
                                                                   long long ss, RingWindow rw,
                                                                   float *__restrict__ x, float c, long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float xo = x[i];
        for (int t = 0; t < m; t++)
            if ((rw.cyc >> t) & 1u) xo = fma(c, ldg(ring + (long long)rw.slot[t] * ss + i), xo);
        x[i] = xo;
    }
}

// One history column from two consecutive residuals: df = (rk - rk1) cf and,
// when h is set, h = c rk1 + hb df (the Richardson pass's rounding).
static __global__ void __launch_bounds__(kReduceThreads) ring_column_kernel(const float *__restrict__ rk1,
                                                                     const float *__restrict__ rk,
                                                                     float *__restrict__ df, float *__restrict__ h,
                                                                     float c, float hb, float cf, long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float a = rk1[i];
        const float dfv = (rk[i] - a) * cf;
        df[i] = dfv;
        if (h) h[i] = fma(hb, dfv, c * a);
    }
}

// x += sum_mask H_j - beta cf (r - rs): the iterate of a lean FP32 solve that
// stopped between extrapolations (its Richardson passes left x out).
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) recur_fold_kernel(int m, T *__restrict__ x,
                                                                    const T *__restrict__ r,
                                                                    const T *__restrict__ rs,
                                                                    const T *__restrict__ h, T beta,
                                                                    T cf, long long n, unsigned mask) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        T ac = T(0);
        for (int j = 0; j < m; j++)
            if ((mask >> j) & 1u) ac = ac + ldg(h + j * n + i);
        x[i] = x[i] + (ac - beta * ((r[i] - rs[i]) * cf));
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
    __shared__ double red[(kReduceThreads / 32) * AccWidth<T>::value];
    if (solve_done(ctrl)) return;
    if (threadIdx.x < m) s[threadIdx.x] = ctrl_s<T>(ctrl, threadIdx.x);
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
    Acc<T> a1[1] = {acc};
    block_reduce_store<1>(a1, red, partials + blockIdx.x);
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) cg_step_kernel(T *__restrict__ x,
                                                                 T *__restrict__ r,
                                                                 const T *__restrict__ d,
                                                                 const T *__restrict__ q,
                                                                 long long n, int restart,
                                                                 double *partials,
                                                                 const DevCtrl *ctrl) {
    __shared__ double red[(kReduceThreads / 32) * AccWidth<T>::value];
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
        Acc<T> a1[1] = {acc};
        block_reduce_store<1>(a1, red, partials + blockIdx.x);
    }
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) norm2_kernel(const T *__restrict__ v, long long n,
                                                               double *partials,
                                                               const DevCtrl *ctrl) {
    __shared__ double red[(kReduceThreads / 32) * AccWidth<T>::value];
    if (solve_done(ctrl)) return;
    Acc<T> acc;
    acc.zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T a = ldg(v + i);
        acc.add_prod(a, a);
    }
    Acc<T> a1[1] = {acc};
    block_reduce_store<1>(a1, red, partials + blockIdx.x * AccWidth<T>::value);
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
                                 const T *x, const T *b, T *r, T *df, T *hc, S cf, double hb,
                                 double *partials, const DevCtrl *ctrl) {
    switch (mode) {
    case RES_INIT: {
        ResidualOp<T, RES_INIT> op{x, b, r, df, nullptr, (T)cf, T(0.0), partials, ctrl};
        return launch_stencil<T>(L, w, op);
    }
    case RES_ANDERSON: {
        ResidualOp<T, RES_ANDERSON> op{x, b, r, df, hc, (T)cf, T(hb), partials, ctrl};
        return launch_stencil<T>(L, w, op);
    }
    default: {
        ResidualOp<T, RES_APPLY> op{x, b, r, df, nullptr, (T)cf, T(0.0), partials, ctrl};
        return launch_stencil<T>(L, w, op);
    }
    }
}

template <typename T>
cudaError_t Kernels<T>::richardson(const StencilLaunch &L, const Weights<T> &w, int mode,
                                   const T *x, const T *r, const T *b, T *x2, T *r2, T *dx,
                                   T *df, S c, S cf, double hb, const DevCtrl *ctrl) {
    if (mode == RICH_AAR) {
        RichOp<T, RICH_AAR> op{x, r, b, x2, r2, dx, df, (T)c, (T)cf, T(hb), nullptr, ctrl};
        return launch_stencil<T>(L, w, op);
    }
    RichOp<T, RICH_PGR> op{x, r, b, x2, r2, dx, df, (T)c, (T)cf, T(0.0), nullptr, ctrl};
    return launch_stencil<T>(L, w, op);
}

template <typename T>
cudaError_t Kernels<T>::richardson_recur(const StencilLaunch &L, const Weights<T> &w, const T *r,
                                         T *x, T *r2, T *dx, T *df, S c, S cf, double hb,
                                         const DevCtrl *ctrl) {
    RichRecurOp<T> op{r, x, r2, dx, df, (T)c, (T)cf, T(hb), nullptr, ctrl};
    return launch_stencil<T>(L, w, op);
}

template <typename T>
cudaError_t Kernels<T>::richardson_lean(const StencilLaunch &L, const Weights<T> &w, const T *r, T *r2,
                                        T *dx, T *df, S c, S cf, double hb, const DevCtrl *ctrl) {
    if constexpr (std::is_same<typename RealOf<T>::type, float>::value) {
        RichLeanOp<T> op{r, r2, dx, df, (T)c, (T)cf, T(hb), nullptr, ctrl};
        return launch_stencil<T>(L, w, op);
    } else {  // FP64 keeps the reference form
        (void)L, (void)w, (void)r, (void)r2, (void)dx, (void)df, (void)c, (void)cf, (void)hb, (void)ctrl;
        return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t Kernels<T>::ring_richardson(const StencilLaunch &L, const Weights<T> &w, const T *r, T *r2, S c,
                                        const DevCtrl *ctrl) {
    if constexpr (std::is_same<T, float>::value) {
        RichRingOp<T> op{r, r2, (T)c, nullptr, ctrl};
        return launch_stencil<T>(L, w, op);
    } else {
        (void)L, (void)w, (void)r, (void)r2, (void)c, (void)ctrl;
        return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t Kernels<T>::ring_residual(const StencilLaunch &L, const Weights<T> &w, const T *step, const T *r,
                                      T *r2, T *hc, S cf, double hb, double *partials, const DevCtrl *ctrl) {
    if constexpr (std::is_same<T, float>::value) {
        ResRingOp<T> op{step, r, r2, hc, (T)cf, T(hb), partials, ctrl};
        return launch_stencil<T>(L, w, op);
    } else {
        (void)L, (void)w, (void)step, (void)r, (void)r2, (void)hc, (void)cf, (void)hb, (void)partials, (void)ctrl;
        return cudaErrorInvalidValue;
    }
}

template <typename T>
long long Kernels<T>::ring_paired_plan(const Geom &g, int *lz) {
    if constexpr (std::is_same<T, float>::value) {
        static int slots = 0;
        if (slots == 0) {
            int occ = 0, dev = 0, sms = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &occ, stencil_x2_kernel<T, kPairBY, kPairNY, kPairMINB, RichRingOp<T>>, 32 * kPairBY, 0) !=
                    cudaSuccess ||
                occ < 1) {
                cudaGetLastError();
                occ = 1;
            }
            slots = std::max(1, sms) * occ;
        }
        const int z = balanced_lz(g, kPairBY * kPairNY, slots, FillCost<T>::value, 64);
        if (lz) *lz = z;
        return (long long)((g.nx + 63) / 64) * ((g.ny + kPairBY * kPairNY - 1) / (kPairBY * kPairNY)) *
               ((g.nz + z - 1) / z);
    } else {
        (void)g;
        if (lz) *lz = 0;
        return 0;
    }
}

template <typename T>
cudaError_t Kernels<T>::residual_recur(const StencilLaunch &L, const Weights<T> &w, const T *step,
                                       T *r, T *df, T *hc, S cf, double hb, double *partials,
                                       const DevCtrl *ctrl) {
    ResRecurOp<T> op{step, r, df, hc, (T)cf, T(hb), partials, ctrl};
    return launch_stencil<T>(L, w, op);
}

// One block's share of the Hermitian Gram sums (2 reals per value).
template <typename R, int M>
__device__ __forceinline__ void gram_c_block(const cplx<R> *__restrict__ df,
                                             const cplx<R> *__restrict__ r, long long n,
                                             double *out, long long blk, long long nblk) {
    constexpr int NP = (M * (M + 1)) / 2;
    constexpr int NV = NP + M;
    __shared__ double red[2 * NV * (kReduceThreads / 32)];
    Acc<cplx<R>> acc[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) acc[k].zero();
    const long long stride = nblk * blockDim.x;
    if constexpr (std::is_same<R, float>::value) {
        // complex64: two points per 16-byte load; the real and imaginary parts
        // of conj(a) b over both points are summed in FP32 (four products each)
        // and then folded into the double-float accumulators, as the real Gram
        // folds its four-point dot products
        if (n % 2 == 0 && aligned16(df, r)) {
            const long long nv = n / 2;
            const float4 *dv = reinterpret_cast<const float4 *>(df);
            const float4 *rvv = reinterpret_cast<const float4 *>(r);
            for (long long i = blk * blockDim.x + threadIdx.x; i < nv; i += stride) {
                float4 f[M];
#pragma unroll
                for (int j = 0; j < M; j++) f[j] = ldg(dv + j * nv + i);
                const float4 rv = ldg(rvv + i);
                auto cdot = [](const float4 &a, const float4 &b, Acc<cplx<float>> &c) {
                    const float re = fmaf(a.w, b.w, fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)));
                    const float im = fmaf(-a.w, b.z, fmaf(a.z, b.w, fmaf(-a.y, b.x, a.x * b.y)));
                    c.re.add(re);
                    c.im.add(im);
                };
                int k = 0;
#pragma unroll
                for (int j = 0; j < M; j++)
#pragma unroll
                    for (int a = 0; a <= j; a++) { cdot(f[a], f[j], acc[k]); k++; }
#pragma unroll
                for (int j = 0; j < M; j++) cdot(f[j], rv, acc[NP + j]);
            }
            block_reduce_store<NV>(acc, red, out);
            return;
        }
    }
    for (long long i = blk * blockDim.x + threadIdx.x; i < n; i += stride) {
        cplx<R> f[M];
#pragma unroll
        for (int j = 0; j < M; j++) f[j] = ldg(df + j * n + i);
        const cplx<R> rv = ldg(r + i);
        int k = 0;
#pragma unroll
        for (int j = 0; j < M; j++)
#pragma unroll
            for (int a = 0; a <= j; a++) { acc[k].add_prod(f[a], f[j]); k++; }
#pragma unroll
        for (int j = 0; j < M; j++) acc[NP + j].add_prod(f[j], rv);
    }
    block_reduce_store<NV>(acc, red, out);
}

// Hermitian Gram for complex vectors (PETSC_COMPLEX/AAR_Complex.c:213-216):
// G(a,j) = DF_a^H DF_j (a <= j), h_j = DF_j^H r; M compile-time history depth.
template <typename R, int M>
__global__ void __launch_bounds__(kReduceThreads) gram_c_kernel(const cplx<R> *__restrict__ df,
                                                                const cplx<R> *__restrict__ r,
                                                                long long n, double *partials,
                                                                const DevCtrl *ctrl) {
    constexpr int NV = (M * (M + 1)) / 2 + M;
    if (solve_done(ctrl)) return;
    gram_c_block<R, M>(df, r, n, partials + (long long)blockIdx.x * 2 * NV, blockIdx.x, gridDim.x);
}

// Generic Hermitian Gram for complex vectors, m > 8: one value per
// (block, value slot), G(a,j) = DF_a^H DF_j (a <= j) or h_j = DF_j^H r, the
// columns re-read per value from L2; partials laid out as gram_c_block's
// (2 reals per value, nv values per block).
template <typename R>
__global__ void __launch_bounds__(kReduceThreads) gram_generic_c_kernel(int m, const cplx<R> *__restrict__ df,
                                                                        const cplx<R> *__restrict__ r, long long n,
                                                                        int nv, double *partials,
                                                                        const DevCtrl *ctrl) {
    __shared__ double red[(kReduceThreads / 32) * 2];
    __shared__ double out[2];
    if (solve_done(ctrl)) return;
    const int v = blockIdx.y;
    const int np = (m * (m + 1)) / 2;
    const cplx<R> *u, *w;
    if (v < np) {
        int j = 0;
        while ((j + 1) * (j + 2) / 2 <= v) j++;
        const int a = v - j * (j + 1) / 2;
        u = df + (long long)a * n;
        w = df + (long long)j * n;
    } else {
        u = df + (long long)(v - np) * n;
        w = r;
    }
    Acc<cplx<R>> acc[1];
    acc[0].zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        acc[0].add_prod(ldg(u + i), ldg(w + i));
    block_reduce_store<1>(acc, red, out);
    __syncthreads();
    if (threadIdx.x < 2) partials[((long long)blockIdx.x * nv + v) * 2 + threadIdx.x] = out[threadIdx.x];
}

template <typename T, int KIND>
static cudaError_t gram_dispatch(int m, const T *dx, const T *df, const T *r, long long n,
                                 double *partials, int blocks, const DevCtrl *ctrl,
                                 cudaStream_t s) {
    const int vn = Vec4<T>::N;
    if constexpr (std::is_same<T, float>::value && KIND == GRAM_SYM) {
        // the bulk-copy form: 16-byte aligned columns and residual, n % 4 == 0
        if (n % 4 == 0 && m >= 1 && m <= 8 && (((uintptr_t)df | (uintptr_t)r) & 15u) == 0) {
            DevCtrl *c = const_cast<DevCtrl *>(ctrl);
            const unsigned extra_tx = gram_fault_tx();
            const long long wait_cycles = gram_wait_cycles();
            switch (m) {
#define LSG_GRAM_BULK(MM)                                                                                     \
    case MM: {                                                                                                \
        /* the attribute is per device and context: set on every launch (a cheap host call) */               \
        const cudaError_t ea = cudaFuncSetAttribute(gram_bulk_kernel<MM>,                                     \
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize,              \
                                                    (int)gram_bulk_smem<MM>());                               \
        if (ea != cudaSuccess) return ea;                                                                     \
        gram_bulk_kernel<MM><<<blocks, kReduceThreads, gram_bulk_smem<MM>(), s>>>(df, r, n, partials, c,      \
                                                                                  extra_tx, wait_cycles);     \
        return cudaGetLastError();                                                                            \
    }
                LSG_GRAM_BULK(1) LSG_GRAM_BULK(2) LSG_GRAM_BULK(3) LSG_GRAM_BULK(4)
                LSG_GRAM_BULK(5) LSG_GRAM_BULK(6) LSG_GRAM_BULK(7) LSG_GRAM_BULK(8)
#undef LSG_GRAM_BULK
            default: break;
            }
        }
    }
    switch (n % vn == 0 && aligned16(dx, df, r) ? m : 0) {
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

// One wave of the Gram kernel: resident blocks per SM x SMs (cached per kind, m).
template <typename T>
int Kernels<T>::gram_grid(int kind, int m, long long n, int sms) {
    static int cache[2][LSG_MAX_M + 1];
    int &occ = cache[kind == GRAM_SYM ? 0 : 1][m];
    if constexpr (IsCplx<T>::value) {
        (void)kind;
        if (occ == 0) occ = 1;
    } else if (occ == 0) {
        int v = 0;
        cudaError_t e = cudaSuccess;
        switch (m) {
#define LSG_GRAM_OCC(MM)                                                                                  \
    case MM:                                                                                              \
        e = kind == GRAM_SYM                                                                              \
                ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, gram_kernel<T, GRAM_SYM, MM>, kReduceThreads, 0) \
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, gram_kernel<T, GRAM_GALERKIN, MM>, kReduceThreads, 0); \
        break;
            LSG_GRAM_OCC(1) LSG_GRAM_OCC(2) LSG_GRAM_OCC(3) LSG_GRAM_OCC(4)
            LSG_GRAM_OCC(5) LSG_GRAM_OCC(6) LSG_GRAM_OCC(7) LSG_GRAM_OCC(8)
#undef LSG_GRAM_OCC
        default: v = 4;
        }
        if (e != cudaSuccess || v < 1) { cudaGetLastError(); v = 2; }
        occ = v;
    }
    const long long need = (n + kReduceThreads - 1) / kReduceThreads;
    return (int)std::max<long long>(1, std::min<long long>(need, (long long)occ * sms));
}

template <typename T>
cudaError_t Kernels<T>::gram(int kind, int m, const T *dx, const T *df, const T *r, long long n,
                             double *partials, int blocks, const DevCtrl *ctrl, cudaStream_t s, int exact) {
    if constexpr (std::is_same<T, double>::value) {
        if (!exact && m >= 1 && m <= 8) {
            DevCtrl *c = const_cast<DevCtrl *>(ctrl);
            switch (m) {
#define LSG_GRAM_DF(MM)                                                                                        \
    case MM:                                                                                                   \
        if (kind == GRAM_SYM)                                                                                  \
            gram_df_kernel<GRAM_SYM, MM><<<blocks, kReduceThreads, 0, s>>>(dx, df, r, n, partials, c);         \
        else                                                                                                   \
            gram_df_kernel<GRAM_GALERKIN, MM><<<blocks, kReduceThreads, 0, s>>>(dx, df, r, n, partials, c);    \
        return cudaGetLastError();
                LSG_GRAM_DF(1) LSG_GRAM_DF(2) LSG_GRAM_DF(3) LSG_GRAM_DF(4)
                LSG_GRAM_DF(5) LSG_GRAM_DF(6) LSG_GRAM_DF(7) LSG_GRAM_DF(8)
#undef LSG_GRAM_DF
            default: break;
            }
        }
    }
    if constexpr (IsCplx<T>::value) {
        using R = typename RealOf<T>::type;
        (void)kind;
        (void)dx;
        switch (m) {
#define LSG_GRAMC_CASE(MM) \
    case MM: gram_c_kernel<R, MM><<<blocks, kReduceThreads, 0, s>>>(df, r, n, partials, ctrl); break;
            LSG_GRAMC_CASE(1) LSG_GRAMC_CASE(2) LSG_GRAMC_CASE(3) LSG_GRAMC_CASE(4)
            LSG_GRAMC_CASE(5) LSG_GRAMC_CASE(6) LSG_GRAMC_CASE(7) LSG_GRAMC_CASE(8)
#undef LSG_GRAMC_CASE
        default: {
            if (m < 1 || 2 * m > LSG_MAX_M) return cudaErrorInvalidValue;
            const int nv = (m * (m + 1)) / 2 + m;
            gram_generic_c_kernel<R><<<dim3(blocks, nv), kReduceThreads, 0, s>>>(m, df, r, n, nv, partials, ctrl);
        }
        }
        return cudaGetLastError();
    } else {
    if (kind == GRAM_SYM) return gram_dispatch<T, GRAM_SYM>(m, dx, df, r, n, partials, blocks, ctrl, s);
    return gram_dispatch<T, GRAM_GALERKIN>(m, dx, df, r, n, partials, blocks, ctrl, s);
    }
}

template <typename T>
cudaError_t Kernels<T>::aar_update_lean(int m, T *x, const T *r, const T *rs, const T *h, T *step,
                                        double beta, S cf, long long n, unsigned mask, const DevCtrl *ctrl,
                                        cudaStream_t s) {
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, (long long)sm_count() * 8);
    if constexpr (!std::is_same<typename RealOf<T>::type, float>::value) {  // FP64 keeps the reference form
        (void)m, (void)x, (void)r, (void)rs, (void)h, (void)step, (void)beta, (void)cf, (void)mask, (void)ctrl,
            (void)s, (void)blocks;
        return cudaErrorInvalidValue;
    } else if constexpr (IsCplx<T>::value) {
        aar_update_lean_kernel<T, 0><<<blocks, kReduceThreads, 0, s>>>(m, x, r, rs, h, step, T(beta), (T)cf, n,
                                                                      mask, ctrl);
    } else {
        const bool vec = n % Vec4<T>::N == 0 && aligned16(x, r, rs, h, step);
        switch (vec ? m : 0) {
#define LSG_UPD_CASE(MM)                                                                                      \
    case MM:                                                                                                  \
        aar_update_lean_kernel<T, MM><<<blocks, kReduceThreads, 0, s>>>(m, x, r, rs, h, step, (T)beta, (T)cf, \
                                                                       n, mask, ctrl);                        \
        break;
            LSG_UPD_CASE(1) LSG_UPD_CASE(2) LSG_UPD_CASE(3) LSG_UPD_CASE(4)
            LSG_UPD_CASE(5) LSG_UPD_CASE(6) LSG_UPD_CASE(7) LSG_UPD_CASE(8)
#undef LSG_UPD_CASE
        default:
            aar_update_lean_kernel<T, 0><<<blocks, kReduceThreads, 0, s>>>(m, x, r, rs, h, step, (T)beta, (T)cf,
                                                                          n, mask, ctrl);
        }
    }
    return cudaGetLastError();
}

// The ring kernels need m <= 8, n % 4 == 0 and 16-byte aligned ring, x, step and history.
template <typename T>
cudaError_t Kernels<T>::ring_gram(int m, const RingWindow &rw, const T *ring, long long ss, const T *df, S cf,
                                  long long n, double *partials, int blocks, DevCtrl *ctrl, cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        if (m < 1 || m > kRingMaxM || n % 4 != 0 || ss % 4 != 0 || !aligned16(ring, df))
            return cudaErrorInvalidValue;
        const unsigned extra_tx = gram_fault_tx();
        const long long wait_cycles = gram_wait_cycles();
        const bool full = rw.valid == (1u << m) - 1u && rw.dfmem == 0u;
        switch (m) {
#define LSG_GRAM_RING(MM)                                                                                   \
    case MM: {                                                                                              \
        auto *kern = full ? gram_bulk_kernel<MM, true, true> : gram_bulk_kernel<MM, true, false>;           \
        const cudaError_t ea = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                                                    (int)gram_bulk_smem<MM>());                             \
        if (ea != cudaSuccess) return ea;                                                                   \
        kern<<<blocks, kReduceThreads, gram_bulk_smem<MM>(), s>>>(df, nullptr, n, partials, ctrl, extra_tx, \
                                                                  wait_cycles, ring, ss, rw, (float)cf);    \
        return cudaGetLastError();                                                                          \
    }
            LSG_GRAM_RING(1) LSG_GRAM_RING(2) LSG_GRAM_RING(3) LSG_GRAM_RING(4)
            LSG_GRAM_RING(5) LSG_GRAM_RING(6) LSG_GRAM_RING(7) LSG_GRAM_RING(8)
#undef LSG_GRAM_RING
        default: return cudaErrorInvalidValue;
        }
    } else {
        (void)m, (void)rw, (void)ring, (void)ss, (void)df, (void)cf, (void)n, (void)partials, (void)blocks,
            (void)ctrl, (void)s;
        return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t Kernels<T>::ring_update(int m, const RingWindow &rw, const T *ring, long long ss, const T *h, T *x,
                                    T *step, S c, double beta, S cf, long long n, const DevCtrl *ctrl,
                                    cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        if (m < 1 || m > kRingMaxM || n % 4 != 0 || ss % 4 != 0 || !aligned16(ring, h, x, step))
            return cudaErrorInvalidValue;
        const long long nb = (n / 4 + kReduceThreads - 1) / kReduceThreads;  // one float4 per thread
        if (nb > 0x7fffffffLL) return cudaErrorInvalidValue;
        const unsigned blocks = (unsigned)nb;
        switch (m) {
#define LSG_UPD_RING(MM)                                                                                     \
    case MM:                                                                                                 \
        aar_update_ring_kernel<MM><<<blocks, kReduceThreads, 0, s>>>(ring, ss, rw, h, x, step, (float)c,     \
                                                                     (float)beta, (float)cf, n, ctrl);       \
        break;
            LSG_UPD_RING(1) LSG_UPD_RING(2) LSG_UPD_RING(3) LSG_UPD_RING(4)
            LSG_UPD_RING(5) LSG_UPD_RING(6) LSG_UPD_RING(7) LSG_UPD_RING(8)
#undef LSG_UPD_RING
        default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    } else {
        (void)m, (void)rw, (void)ring, (void)ss, (void)h, (void)x, (void)step, (void)c, (void)beta, (void)cf, (void)n,
            (void)ctrl, (void)s;
        return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t Kernels<T>::ring_fold(int m, const RingWindow &rw, const T *ring, long long ss, T *x, S c, long long n,
                                  cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, (long long)sm_count() * 8);
        ring_fold_kernel<<<blocks, kReduceThreads, 0, s>>>(m, ring, ss, rw, x, (float)c, n);
        return cudaGetLastError();
    } else {
        (void)m, (void)rw, (void)ring, (void)ss, (void)x, (void)c, (void)n, (void)s;
        return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t Kernels<T>::ring_store_column(const T *rk1, const T *rk, T *df, T *h, S c, double hb, S cf,
                                          long long n, cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, (long long)sm_count() * 8);
        ring_column_kernel<<<blocks, kReduceThreads, 0, s>>>(rk1, rk, df, h, (float)c, (float)hb, (float)cf, n);
        return cudaGetLastError();
    } else {
        (void)rk1, (void)rk, (void)df, (void)h, (void)c, (void)hb, (void)cf, (void)n, (void)s;
        return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t Kernels<T>::recur_fold(int m, T *x, const T *r, const T *rs, const T *h, double beta, S cf,
                                   long long n, unsigned mask, cudaStream_t s) {
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, (long long)sm_count() * 8);
    if constexpr (!std::is_same<typename RealOf<T>::type, float>::value) {
        (void)m, (void)x, (void)r, (void)rs, (void)h, (void)beta, (void)cf, (void)mask, (void)s, (void)blocks;
        return cudaErrorInvalidValue;
    } else {
        recur_fold_kernel<T><<<blocks, kReduceThreads, 0, s>>>(m, x, r, rs, h, T(beta), (T)cf, n, mask);
        return cudaGetLastError();
    }
}

template <typename T>
cudaError_t Kernels<T>::aar_update(int m, T *x, const T *r, const T *h, T *step, double beta,
                                   S cf, long long n, const DevCtrl *ctrl, cudaStream_t s) {
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, (long long)sm_count() * 8);
    if constexpr (IsCplx<T>::value) {
        aar_update_kernel<T, 0><<<blocks, kReduceThreads, 0, s>>>(m, x, r, h, step, T(beta), (T)cf, n, ctrl);
    } else {
        // 16-byte loads need every vector 16-byte aligned (x may be a view at an element offset)
        const bool vec = n % Vec4<T>::N == 0 && aligned16(x, r, h, step);
        switch (vec ? m : 0) {
#define LSG_UPD_CASE(MM) \
    case MM: aar_update_kernel<T, MM><<<blocks, kReduceThreads, 0, s>>>(m, x, r, h, step, (T)beta, (T)cf, n, ctrl); break;
            LSG_UPD_CASE(1) LSG_UPD_CASE(2) LSG_UPD_CASE(3) LSG_UPD_CASE(4)
            LSG_UPD_CASE(5) LSG_UPD_CASE(6) LSG_UPD_CASE(7) LSG_UPD_CASE(8)
#undef LSG_UPD_CASE
        default: aar_update_kernel<T, 0><<<blocks, kReduceThreads, 0, s>>>(m, x, r, h, step, (T)beta, (T)cf, n, ctrl);
        }
    }
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
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, (long long)sm_count() * 8);
    axpy_kernel<T><<<blocks, kReduceThreads, 0, s>>>(x, y, (T)alpha, n);
    return cudaGetLastError();
}

template <typename T64, typename T32>
cudaError_t ir_residual(const StencilLaunch &L, const Weights<T64> &w, const T64 *x,
                        const T64 *b, T32 *r32, double *partials, const DevCtrl *ctrl, int zgate) {
    IrResidualOp<T64, T32> op{x, b, r32, partials, ctrl, zgate};
    return launch_stencil<T64>(L, w, op);
}

template <typename T64, typename T32>
__global__ void __launch_bounds__(kReduceThreads) ir_residual_const_kernel(const T64 *__restrict__ b,
                                                                           T32 *__restrict__ r32, long long n,
                                                                           double *partials, const DevCtrl *ctrl,
                                                                           double sr, double si) {
    constexpr int W = AccWidth<T64>::value;
    __shared__ double red[(kReduceThreads / 32) * W];
    if (solve_done(ctrl) || !ctrl->x_zero) return;
    T64 c;  // sigma * shift
    if constexpr (IsCplx<T64>::value)
        c = T64(sr * ctrl->shift[0] - si * ctrl->shift[1], sr * ctrl->shift[1] + si * ctrl->shift[0]);
    else
        c = sr * ctrl->shift[0];
    Acc<T64> acc;
    acc.zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const T64 rn = ldg(b + i) - c;
        r32[i] = (T32)rn;
        acc.add_prod(rn, rn);
    }
    Acc<T64> a1[1] = {acc};
    block_reduce_store<1>(a1, red, partials + (long long)blockIdx.x * W);
}

template <typename T64, typename T32>
cudaError_t ir_residual_const(const T64 *b, T32 *r32, long long n, double *partials, int blocks,
                              const DevCtrl *ctrl, double sig_re, double sig_im, cudaStream_t s) {
    ir_residual_const_kernel<T64, T32><<<blocks, kReduceThreads, 0, s>>>(b, r32, n, partials, ctrl, sig_re, sig_im);
    return cudaGetLastError();
}

template <typename T64>
__global__ void __launch_bounds__(kReduceThreads) zero_check_kernel(const T64 *__restrict__ x, long long n,
                                                                    DevCtrl *ctrl) {
    bool nz = false;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if constexpr (IsCplx<T64>::value) {
            const T64 v = x[i];
            nz |= (v.x != 0.0) || (v.y != 0.0);
        } else {
            nz |= x[i] != 0.0;  // NaN counts as non-zero
        }
    }
    if (__syncthreads_or(nz) && threadIdx.x == 0) ctrl->x_zero = 0;
}

template <typename T64>
cudaError_t zero_check(const T64 *x, long long n, DevCtrl *ctrl, cudaStream_t s) {
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, (long long)sm_count() * 4);
    zero_check_kernel<T64><<<blocks, kReduceThreads, 0, s>>>(x, n, ctrl);
    return cudaGetLastError();
}

// x64 += e32; e32 = 0 (the correction is folded into x and restarts at zero).
template <typename T64, typename T32>
__global__ void ir_correct_kernel(T64 *__restrict__ x, T32 *__restrict__ e, long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        x[i] += (T64)e[i];
        e[i] = T32(0.0);
    }
}

// ---- constant-mode deflation (mixed solves)
template <typename T64>
__global__ void __launch_bounds__(kReduceThreads) mean_sum_kernel(const T64 *__restrict__ v, long long n,
                                                                  double *partials) {
    __shared__ double red[2 * (kReduceThreads / 32)];
    double re = 0.0, im = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if constexpr (IsCplx<T64>::value) {
            const T64 u = v[i];
            re += u.x;
            im += u.y;
        } else {
            re += v[i];
        }
    }
    Acc<double> acc[2];
    acc[0].v = re;
    acc[1].v = im;
    block_reduce_store<2>(acc, red, partials + 2 * (long long)blockIdx.x);
}

// which 0: ctrl->bmean = the mean; 1: ctrl->shift = bmean / sigma - the mean
static __global__ void mean_finalize_kernel(const double *partials, int nparts, long long n, DevCtrl *ctrl, int which,
                                     double sr, double si) {
    __shared__ double red[2 * (kReduceThreads / 32)];
    double re = 0.0, im = 0.0;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
        re += partials[2 * k];
        im += partials[2 * k + 1];
    }
    Acc<double> acc[2];
    acc[0].v = re;
    acc[1].v = im;
    __shared__ double out[2];
    block_reduce_store<2>(acc, red, out);
    __syncthreads();
    if (threadIdx.x != 0) return;
    const double mr = out[0] / (double)n, mi = out[1] / (double)n;
    if (which == 0) {
        ctrl->bmean[0] = mr;
        ctrl->bmean[1] = mi;
    } else {
        const double d = sr * sr + si * si;
        const double br = ctrl->bmean[0], bi = ctrl->bmean[1];
        ctrl->shift[0] = (br * sr + bi * si) / d - mr;
        ctrl->shift[1] = (bi * sr - br * si) / d - mi;
    }
}

template <typename T64>
__global__ void __launch_bounds__(kReduceThreads) shift_kernel(T64 *__restrict__ x, long long n,
                                                               const DevCtrl *ctrl) {
    T64 c;
    if constexpr (IsCplx<T64>::value) c = T64(ctrl->shift[0], ctrl->shift[1]);
    else c = ctrl->shift[0];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) x[i] = x[i] + c;
}

template <typename T64>
cudaError_t rhs_mean(const T64 *b, long long n, double *partials, DevCtrl *ctrl, cudaStream_t s) {
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, (long long)sm_count() * 4);
    mean_sum_kernel<T64><<<blocks, kReduceThreads, 0, s>>>(b, n, partials);
    mean_finalize_kernel<<<1, kReduceThreads, 0, s>>>(partials, blocks, n, ctrl, 0, 0.0, 0.0);
    return cudaGetLastError();
}

template <typename T64>
cudaError_t deflate_x(T64 *x, long long n, double *partials, DevCtrl *ctrl, double sig_re, double sig_im,
                      cudaStream_t s) {
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, (long long)sm_count() * 4);
    mean_sum_kernel<T64><<<blocks, kReduceThreads, 0, s>>>(x, n, partials);
    mean_finalize_kernel<<<1, kReduceThreads, 0, s>>>(partials, blocks, n, ctrl, 1, sig_re, sig_im);
    shift_kernel<T64><<<blocks, kReduceThreads, 0, s>>>(x, n, ctrl);
    return cudaGetLastError();
}

template <typename T64, typename T32>
cudaError_t ir_correct(T64 *x, T32 *e, long long n, cudaStream_t s) {
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, (long long)sm_count() * 8);
    ir_correct_kernel<T64, T32><<<blocks, kReduceThreads, 0, s>>>(x, e, n);
    return cudaGetLastError();
}

}  // namespace lsg
