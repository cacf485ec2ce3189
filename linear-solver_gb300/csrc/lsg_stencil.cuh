// lsg_stencil.cuh — z-marching periodic star-stencil driver.
//
// Replaces the sequential operator of MPI_REAL/system.c:189-204 (and the MPI
// halo exchange of :106-188, which one GPU does not need): each thread block
// owns a 32 x TY column tile of the xy plane (NY adjacent rows per thread) and a
// range of lz planes along z.
// For every plane it
//   * keeps, per owned column, the 2R+1 values u(z-R .. z+R) in a register
//     queue (one new plane value loaded per step: the z neighbours),
//   * stages plane z with an R-wide xy halo in shared memory (the interior
//     from the queue centre, the halo from global memory; the periodic wrap
//     of the xy coordinates is computed once, before the march),
//   * evaluates Au = w0 u_c + sum_p w_p ((u_x-p + u_x+p) + (u_y-p + u_y+p) + (u_z-p + u_z+p)),
// while the global loads of plane z+1 (queue head, halo, centre operands) are
// already in flight.  The shared plane is double-buffered, so one barrier per
// plane suffices.
//
// The value u at a grid point and what happens to Au at the centre are
// supplied by a functor, so one driver serves every stencil pass.
// Functor interface (all __device__):
//   bool skip() const                     the solve has finished: return at once
//   void init()                           read device scalars (once per thread)
//   Raw  fetch(unsigned idx) const        global loads for u at idx
//   T    value(const Raw &) const         u from the fetched operands
//   Ctr  fetch_center(unsigned idx) const operands the epilogue needs at a centre
//   void store(unsigned idx, T u, T Au, const Ctr &, Acc<T> *acc) const
// Flat indices are 32-bit: grids are limited to 2^32 - 1 points.
//   static constexpr int NACC             per-thread accumulators reduced per block
//   double *partials                      where the block writes NACC sums
#pragma once

#include <cstring>
#include <type_traits>

#include "lsg_internal.cuh"
#include "lsg_accum.cuh"
#include "lsg_complex.cuh"
#include "lsg_df.cuh"

namespace lsg {

template <typename T>
__device__ __forceinline__ T ldg(const T *p) { return __ldg(p); }

struct NoCtr {};

// Bounds-checked build (-DLSG_BOUNDS): every global and shared index of the
// stencil marches is checked; the first out-of-range index is recorded
// (+1, in this translation unit's word) and the access is skipped (a load
// reads element 0 instead).  lsg_bounds_errors() reads the words of every
// unit.  The normal build compiles the checks away.
#ifdef LSG_BOUNDS
static __device__ unsigned long long g_bounds_bad;
__device__ __forceinline__ bool bounds_ok(unsigned long long i, unsigned long long n) {
    if (i < n) return true;
    atomicCAS(&g_bounds_bad, 0ull, i + 1ull);
    return false;
}
__device__ __forceinline__ unsigned bounds_ix(unsigned long long i, unsigned long long n) {
    return bounds_ok(i, n) ? (unsigned)i : 0u;
}
int register_bounds_reader(unsigned long long (*read)());
static unsigned long long bounds_read_unit() {
    unsigned long long v = 0;
    if (cudaMemcpyFromSymbol(&v, g_bounds_bad, sizeof(v)) != cudaSuccess) cudaGetLastError();
    return v;
}
static const int g_bounds_registered = register_bounds_reader(&bounds_read_unit);
#define LSG_IX(i, n) ::lsg::bounds_ix((unsigned long long)(i), (unsigned long long)(n))
#define LSG_IX_OK(i, n) ::lsg::bounds_ok((unsigned long long)(i), (unsigned long long)(n))
#else
#define LSG_IX(i, n) (i)
#define LSG_IX_OK(i, n) true
#endif

// Calls f(integral_constant<P>), f(integral_constant<P+1>), ... up to Q-1
// while f returns true; returns false as soon as one call does.
template <int P, int Q, class F>
__device__ __forceinline__ bool unrolled_steps(F &f) {
    if constexpr (P < Q) {
        if (!f(std::integral_constant<int, P>{})) return false;
        return unrolled_steps<P + 1, Q>(f);
    } else {
        return true;
    }
}

// RQ: radius the storage is sized for; the arithmetic uses `radius` (== RQ on
// the specialised path, <= RQ on the generic path).
// (bx, by, bz): the block's tile (x, y) and z chunk; blk: where its partial sums go.
template <typename T, int RQ, int BY, int NY, bool GENERIC, class Op>
__device__ __forceinline__ void stencil_march(const Geom &g, const Weights<T> &w, int lz, Op &op,
                                              T *smem0, T *smem1, int bx, int by, int bz,
                                              long long blk) {
    using Raw = typename Op::Raw;
    using Ctr = typename Op::Ctr;
    constexpr int TX = 32;
    constexpr int TY = BY * NY;
    constexpr int FX = TX + 2 * RQ;
    constexpr int NT = 32 * BY;
    constexpr int H = 2 * RQ * TX + TY * 2 * RQ;  // halo cells of one plane (no corners: the stencil is a star)
    constexpr int NH = (H + NT - 1) / NT;
    constexpr int Q = 2 * RQ + 1;
    constexpr int FY = TY + 2 * RQ;
    const unsigned long long gn = (unsigned long long)g.n;
    (void)gn;

    const int radius = GENERIC ? w.radius : RQ;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tx;
    const int x0 = bx * TX, y0 = by * TY;
    const int z0 = bz * lz;
    const int z1 = min(z0 + lz, g.nz);

    // Owned columns (periodically wrapped, so partial tiles still hold valid data).
    const int gx = wrap_index(x0 + tx, g.nx);
    int col[NY];
    bool valid[NY];
#pragma unroll
    for (int k = 0; k < NY; k++) {
        const int yy = y0 + ty * NY + k;  // a thread owns NY adjacent rows
        col[k] = gx + wrap_index(yy, g.ny) * g.nx;
        valid[k] = (x0 + tx < g.nx) && (yy < g.ny);
    }
    // Halo cells this thread fills, as (shared offset, wrapped xy offset).
    int hs[NH], ho[NH];
#pragma unroll
    for (int s = 0; s < NH; s++) {
        const int h = tid + s * NT;
        hs[s] = -1;
        ho[s] = 0;
        if (h < H) {
            int fy, fx;
            if (h < RQ * TX) {                       // top strip
                fy = h / TX; fx = RQ + h % TX;
            } else if (h < 2 * RQ * TX) {            // bottom strip
                const int hh = h - RQ * TX;
                fy = RQ + TY + hh / TX; fx = RQ + hh % TX;
            } else {                                 // left / right strips
                const int hh = h - 2 * RQ * TX;
                const int row = hh / (2 * RQ), c = hh % (2 * RQ);
                fy = RQ + row;
                fx = c < RQ ? c : TX + c;
            }
            hs[s] = fy * FX + fx;
            ho[s] = wrap_index(x0 - RQ + fx, g.nx) + wrap_index(y0 - RQ + fy, g.ny) * g.nx;
        }
    }

    Acc<T> acc[Op::NACC > 0 ? Op::NACC : 1];
#pragma unroll
    for (int a = 0; a < (Op::NACC > 0 ? Op::NACC : 1); a++) acc[a].zero();

    // The register queue is a ring: at phase P (= step index mod Q) slot j
    // holds plane z - RQ + ((j - P) mod Q).  The march is unrolled Q times so
    // every slot index is a compile-time constant and advancing the ring
    // costs no register moves.
    T q[NY][Q];
    // Prologue: planes z0-RQ .. z0+RQ-1 into slots 0..2RQ-1.
    unsigned zl = (unsigned)wrap_index(z0 - RQ, g.nz);
    const unsigned nxy = (unsigned)g.nxy, nz = (unsigned)g.nz;
#pragma unroll
    for (int s = 0; s < 2 * RQ; s++) {
        const unsigned base = zl * nxy;
#pragma unroll
        for (int k = 0; k < NY; k++) q[k][s] = op.value(op.fetch(LSG_IX(base + col[k], gn)));
        zl = (zl + 1 == nz) ? 0u : zl + 1;
    }
    // In flight for the next plane: queue head (plane z+RQ), halo and centres (plane z).
    Raw qn[NY], hn[NH];
    Ctr cn[NY];
    {
        const unsigned lb = zl * nxy, zb = (unsigned)z0 * nxy;
#pragma unroll
        for (int k = 0; k < NY; k++) {
            qn[k] = op.fetch(LSG_IX(lb + col[k], gn));
            cn[k] = op.fetch_center(LSG_IX(zb + col[k], gn));
        }
#pragma unroll
        for (int s = 0; s < NH; s++)
            if (hs[s] >= 0) hn[s] = op.fetch(LSG_IX(zb + ho[s], gn));
        zl = (zl + 1 == nz) ? 0u : zl + 1;
    }

    T *sm = smem0;
    int z = z0;
    auto step = [&](auto phase) -> bool {
        constexpr int P = decltype(phase)::value;
        constexpr int HEAD = (P + Q - 1) % Q;  // slot receiving plane z+RQ
        constexpr int CEN = (P + RQ) % Q;      // slot of plane z
        const unsigned zbase = (unsigned)z * nxy;
#pragma unroll
        for (int k = 0; k < NY; k++) {
            q[k][HEAD] = op.value(qn[k]);
            sm[LSG_IX((RQ + ty * NY + k) * FX + RQ + tx, FX * FY)] = q[k][CEN];
        }
#pragma unroll
        for (int s = 0; s < NH; s++)
            if (hs[s] >= 0) sm[LSG_IX(hs[s], FX * FY)] = op.value(hn[s]);
        Ctr cc[NY];
#pragma unroll
        for (int k = 0; k < NY; k++) cc[k] = cn[k];
        if (z + 1 < z1) {  // issue plane z+1's loads before computing plane z
            const unsigned lb = zl * nxy, nb = zbase + nxy;
#pragma unroll
            for (int k = 0; k < NY; k++) {
                qn[k] = op.fetch(LSG_IX(lb + col[k], gn));
                cn[k] = op.fetch_center(LSG_IX(nb + col[k], gn));
            }
#pragma unroll
            for (int s = 0; s < NH; s++)
                if (hs[s] >= 0) hn[s] = op.fetch(LSG_IX(nb + ho[s], gn));
            zl = (zl + 1 == nz) ? 0u : zl + 1;
        }
        __syncthreads();  // plane z staged; the other buffer is no longer read
        // y neighbours of the thread's NY adjacent rows, rows r0-RQ .. r0+NY-1+RQ:
        // loaded from the staged plane once for all NY points (its own rows
        // are the queue centres), so a point costs 2 RQ + 2 RQ / NY shared loads.
        const T *col0 = sm + (RQ + ty * NY) * FX + RQ + tx;
        T yv[NY + 2 * RQ];
#pragma unroll
        for (int j = 0; j < RQ; j++) {
            yv[j] = col0[(j - RQ) * FX];
            yv[RQ + NY + j] = col0[(NY + j) * FX];
        }
#pragma unroll
        for (int k = 0; k < NY; k++) yv[RQ + k] = q[k][CEN];
#pragma unroll
        for (int k = 0; k < NY; k++) {
            const T *row = col0 + k * FX;
            T au = w.w[0] * q[k][CEN];
#pragma unroll
            for (int p = 1; p <= RQ; p++) {
                if (GENERIC && p > radius) break;
                const T sxy = (row[-p] + row[p]) + (yv[RQ + k - p] + yv[RQ + k + p]);
                const T sz = q[k][(CEN + Q - p) % Q] + q[k][(CEN + p) % Q];
                au = fma(w.w[p], sxy + sz, au);
            }
            if (valid[k] && LSG_IX_OK(zbase + col[k], gn)) op.store(zbase + col[k], q[k][CEN], au, cc[k], acc);
        }
        sm = (sm == smem0) ? smem1 : smem0;
        return ++z < z1;
    };
    while (z < z1) {
        if (!unrolled_steps<0, Q>(step)) break;
    }

    if (Op::NACC > 0) {
        constexpr int NA = Op::NACC > 0 ? Op::NACC : 1;
        constexpr int W = AccWidth<T>::value;
        __shared__ double red[NA * W * 32];
        block_reduce_store<NA>(acc, red, op.partials + blk * Op::NACC * W);
    }
}

// ---------------------------------------------------------------- FP64 in double-float
//
// The march above for FP64 and complex128 vectors with the sums evaluated in
// double-float arithmetic on the FP32 pipe (lsg_df.cuh): the register ring and
// the staged plane hold (hi, lo) float pairs (one per part for complex128,
// DfMarch below), formed once per value with integer and FP32 operations; Au
// is formed with error-free TwoSum / FMA two-product steps.  Each point's sum
// is evaluated in the same order in every tile shape, so results do not
// depend on the launch shape.  Functors opt in with
// DF = true and carry the solve's control block (the split's scale 2^k comes
// from its ||b||; a value beyond the float range sets its df_range flag).
// The ring advances by register moves instead of a Q-fold unrolled march:
// one double-float step is ~10x an FP32 step in code, and the unrolled march
// overflows the instruction cache.

template <class Op, class = void> struct DfOk { static constexpr bool value = false; };
template <class Op> struct DfOk<Op, std::void_t<decltype(Op::DF)>> { static constexpr bool value = Op::DF; };

template <class Op>
__device__ __forceinline__ int df_shift_of(const Op &op) {
    return op.ctrl ? df_shift_for(op.ctrl->rhs_norm) : 0;
}

// VALUE_DF: the functor forms u from its operands in double-float arithmetic
// (value_df(raw, k, bad) -> the pair of u 2^k); the others return a double
// that the march splits.
template <class Op, class = void> struct HasValueDf { static constexpr bool value = false; };
template <class Op>
struct HasValueDf<Op, std::void_t<decltype(Op::VALUE_DF)>> { static constexpr bool value = Op::VALUE_DF; };

// The value the march carries: a (hi, lo) pair for FP64 vectors, a pair per
// part for complex128.  The weights are real but for the centre's, which
// carries the complex shift (w.wfi).  The FP64 steps are the float operations
// of the real march; the complex ones apply them to each part.
__device__ __forceinline__ float2 df_mul3(float2 c, const float *w) {  // c (w[0] + w[1] + w[2])
    float2 au;
    au.x = __fmul_rn(c.x, w[0]);
    au.y = __fmaf_rn(c.x, w[0], -au.x);
    au.y = __fmaf_rn(c.x, w[1], au.y);
    au.y = __fmaf_rn(c.y, w[0], au.y);
    au.y = __fmaf_rn(c.x, w[2], au.y);
    return au;
}

struct DfCplx { float2 re, im; };

template <typename TS> struct DfMarch;
template <> struct DfMarch<double> {
    using V = float2;
    __device__ static __forceinline__ V split(double u, int k, bool &bad) { return df_split(u, k, bad); }
    __device__ static __forceinline__ V add(V a, V b) { return df_add2(a, b); }
    __device__ static __forceinline__ V centre(V c, const Weights<double> &w) { return df_mul3(c, w.wf); }
    __device__ static __forceinline__ void fma_acc(V &au, V s, const float *w3) {
        df_fma_acc(au, s.x, s.y, w3[0], w3[1], w3[2]);
    }
    __device__ static __forceinline__ double to_double(V v, int k) { return df_to_double(v, k); }
};
template <> struct DfMarch<cplx<double>> {
    using V = DfCplx;
    __device__ static __forceinline__ V split(cplx<double> u, int k, bool &bad) {
        return V{df_split(u.x, k, bad), df_split(u.y, k, bad)};
    }
    __device__ static __forceinline__ V add(V a, V b) { return V{df_add2(a.re, b.re), df_add2(a.im, b.im)}; }
    // (c.re + i c.im)(w0 + i w0i): Re = c.re w0 - c.im w0i, Im = c.im w0 + c.re w0i
    __device__ static __forceinline__ V centre(V c, const Weights<cplx<double>> &w) {
        V au{df_mul3(c.re, w.wf), df_mul3(c.im, w.wf)};
        df_fma_acc(au.re, -c.im.x, -c.im.y, w.wfi[0], w.wfi[1], w.wfi[2]);
        df_fma_acc(au.im, c.re.x, c.re.y, w.wfi[0], w.wfi[1], w.wfi[2]);
        return au;
    }
    __device__ static __forceinline__ void fma_acc(V &au, V s, const float *w3) {
        df_fma_acc(au.re, s.re.x, s.re.y, w3[0], w3[1], w3[2]);
        df_fma_acc(au.im, s.im.x, s.im.y, w3[0], w3[1], w3[2]);
    }
    __device__ static __forceinline__ cplx<double> to_double(V v, int k) {
        return cplx<double>(df_to_double(v.re, k), df_to_double(v.im, k));
    }
};
template <typename TS> struct IsDfMarch { static constexpr bool value = false; };
template <> struct IsDfMarch<double> { static constexpr bool value = true; };
template <> struct IsDfMarch<cplx<double>> { static constexpr bool value = true; };

template <typename TS, class Op, class Raw>
__device__ __forceinline__ typename DfMarch<TS>::V df_value(const Op &op, const Raw &v, int k, bool &bad) {
    if constexpr (HasValueDf<Op>::value) return op.value_df(v, k, bad);
    else return DfMarch<TS>::split(op.value(v), k, bad);
}

// STORE_DF: the functor's epilogue takes the centre u and Au as pairs scaled
// by 2^k (store_df(idx, u, Au, ctr, k, acc)); the others get doubles.
template <class Op, class = void> struct HasStoreDf { static constexpr bool value = false; };
template <class Op>
struct HasStoreDf<Op, std::void_t<decltype(Op::STORE_DF)>> { static constexpr bool value = Op::STORE_DF; };

// Operands in flight across the march's loop are carried as integer words:
// loop-carried double registers are copied through the FP64 pipe at the
// loop's back edge, integer ones through the integer pipe.
template <class V, bool BOX = (sizeof(V) % 8 == 0)> struct Bits { V v; };
template <class V> struct Bits<V, true> { unsigned long long w[sizeof(V) / 8]; };
template <class V>
__device__ __forceinline__ Bits<V> to_bits(const V &v) {
    Bits<V> b;
    memcpy(&b, &v, sizeof(V));
    return b;
}
template <class V>
__device__ __forceinline__ V from_bits(const Bits<V> &b) {
    V v;
    memcpy(&v, &b, sizeof(V));
    return v;
}

template <int RQ, int BY, int NY, bool GENERIC, class Op, typename TS>
__device__ __forceinline__ void stencil_march_df(const Geom &g, const Weights<TS> &w, int lz, Op &op,
                                                 TS *smem0d, TS *smem1d, int bx, int by, int bz,
                                                 long long blk) {
    using Raw = typename Op::Raw;
    using Ctr = typename Op::Ctr;
    using DM = DfMarch<TS>;
    using V = typename DM::V;
    static_assert(sizeof(V) == sizeof(TS), "a staged value keeps the vector type's size");
    constexpr int TX = 32;
    constexpr int TY = BY * NY;
    constexpr int FX = TX + 2 * RQ;
    constexpr int NT = 32 * BY;
    constexpr int H = 2 * RQ * TX + TY * 2 * RQ;  // halo cells of one plane (no corners)
    constexpr int NH = (H + NT - 1) / NT;
    constexpr int Q = 2 * RQ + 1;
    constexpr int FY = TY + 2 * RQ;
    const unsigned long long gn = (unsigned long long)g.n;
    (void)gn;
    V *const smem0 = reinterpret_cast<V *>(smem0d);
    V *const smem1 = reinterpret_cast<V *>(smem1d);

    const int radius = GENERIC ? w.radius : RQ;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tx;
    const int x0 = bx * TX, y0 = by * TY;
    const int z0 = bz * lz;
    const int z1 = min(z0 + lz, g.nz);
    const int ks = df_shift_of(op);
    bool bad = false;

    const int gx = wrap_index(x0 + tx, g.nx);
    int col[NY];
    bool valid[NY];
#pragma unroll
    for (int k = 0; k < NY; k++) {
        const int yy = y0 + ty * NY + k;
        col[k] = gx + wrap_index(yy, g.ny) * g.nx;
        valid[k] = (x0 + tx < g.nx) && (yy < g.ny);
    }
    int hs[NH], ho[NH];
#pragma unroll
    for (int s = 0; s < NH; s++) {
        const int h = tid + s * NT;
        hs[s] = -1;
        ho[s] = 0;
        if (h < H) {
            int fy, fx;
            if (h < RQ * TX) {
                fy = h / TX; fx = RQ + h % TX;
            } else if (h < 2 * RQ * TX) {
                const int hh = h - RQ * TX;
                fy = RQ + TY + hh / TX; fx = RQ + hh % TX;
            } else {
                const int hh = h - 2 * RQ * TX;
                const int row = hh / (2 * RQ), c = hh % (2 * RQ);
                fy = RQ + row;
                fx = c < RQ ? c : TX + c;
            }
            hs[s] = fy * FX + fx;
            ho[s] = wrap_index(x0 - RQ + fx, g.nx) + wrap_index(y0 - RQ + fy, g.ny) * g.nx;
        }
    }

    Acc<TS> acc[Op::NACC > 0 ? Op::NACC : 1];
#pragma unroll
    for (int a = 0; a < (Op::NACC > 0 ? Op::NACC : 1); a++) acc[a].zero();

    // ring: q[k][j] holds plane z - RQ + j at the step of plane z
    V q[NY][Q];
    unsigned zl = (unsigned)wrap_index(z0 - RQ, g.nz);
    const unsigned nxy = (unsigned)g.nxy, nz = (unsigned)g.nz;
#pragma unroll
    for (int s = 0; s < 2 * RQ; s++) {
        const unsigned base = zl * nxy;
#pragma unroll
        for (int k = 0; k < NY; k++) q[k][s] = df_value<TS>(op, op.fetch(LSG_IX(base + col[k], gn)), ks, bad);
        zl = (zl + 1 == nz) ? 0u : zl + 1;
    }
    Bits<Raw> qn[NY], hn[NH];
    Bits<Ctr> cn[NY];
    {
        const unsigned lb = zl * nxy, zb = (unsigned)z0 * nxy;
#pragma unroll
        for (int k = 0; k < NY; k++) {
            qn[k] = to_bits(op.fetch(LSG_IX(lb + col[k], gn)));
            cn[k] = to_bits(op.fetch_center(LSG_IX(zb + col[k], gn)));
        }
#pragma unroll
        for (int s = 0; s < NH; s++)
            if (hs[s] >= 0) hn[s] = to_bits(op.fetch(LSG_IX(zb + ho[s], gn)));
        zl = (zl + 1 == nz) ? 0u : zl + 1;
    }

    V *sm = smem0;
#pragma unroll 1
    for (int z = z0; z < z1; z++) {
        constexpr int HEAD = Q - 1;
        constexpr int CEN = RQ;
        const unsigned zbase = (unsigned)z * nxy;
#pragma unroll
        for (int k = 0; k < NY; k++) {
            q[k][HEAD] = df_value<TS>(op, from_bits(qn[k]), ks, bad);
            sm[LSG_IX((RQ + ty * NY + k) * FX + RQ + tx, FX * FY)] = q[k][CEN];
        }
#pragma unroll
        for (int s = 0; s < NH; s++)
            if (hs[s] >= 0) sm[LSG_IX(hs[s], FX * FY)] = df_value<TS>(op, from_bits(hn[s]), ks, bad);
        Bits<Ctr> cc[NY];
#pragma unroll
        for (int k = 0; k < NY; k++) cc[k] = cn[k];
        if (z + 1 < z1) {  // plane z+1's loads in flight while plane z is computed
            const unsigned lb = zl * nxy, nb = zbase + nxy;
#pragma unroll
            for (int k = 0; k < NY; k++) {
                qn[k] = to_bits(op.fetch(LSG_IX(lb + col[k], gn)));
                cn[k] = to_bits(op.fetch_center(LSG_IX(nb + col[k], gn)));
            }
#pragma unroll
            for (int s = 0; s < NH; s++)
                if (hs[s] >= 0) hn[s] = to_bits(op.fetch(LSG_IX(nb + ho[s], gn)));
            zl = (zl + 1 == nz) ? 0u : zl + 1;
        }
        __syncthreads();
        const V *col0 = sm + (RQ + ty * NY) * FX + RQ + tx;
        V yv[NY + 2 * RQ];
#pragma unroll
        for (int j = 0; j < RQ; j++) {
            yv[j] = col0[(j - RQ) * FX];
            yv[RQ + NY + j] = col0[(NY + j) * FX];
        }
#pragma unroll
        for (int k = 0; k < NY; k++) yv[RQ + k] = q[k][CEN];
#pragma unroll
        for (int k = 0; k < NY; k++) {
            const V *row = col0 + k * FX;
            const V c = q[k][CEN];
            V au = DM::centre(c, w);
#pragma unroll
            for (int p = 1; p <= RQ; p++) {
                if (GENERIC && p > radius) break;
                // the six neighbours at distance p, summed as a tree (depth 3)
                const V sx = DM::add(row[-p], row[p]);
                const V sy = DM::add(yv[RQ + k - p], yv[RQ + k + p]);
                const V sz = DM::add(q[k][CEN - p], q[k][CEN + p]);
                const V sp = DM::add(DM::add(sx, sy), sz);
                DM::fma_acc(au, sp, w.wf + 3 * p);
            }
            if (valid[k] && LSG_IX_OK(zbase + col[k], gn)) {
                if constexpr (HasStoreDf<Op>::value)
                    op.store_df(zbase + col[k], c, au, from_bits(cc[k]), ks, acc);
                else
                    op.store(zbase + col[k], DM::to_double(c, ks), DM::to_double(au, ks), from_bits(cc[k]), acc);
            }
        }
        sm = (sm == smem0) ? smem1 : smem0;
        // advance the ring: planes z-RQ+1 .. z+RQ into slots 0 .. 2RQ-1
#pragma unroll
        for (int k = 0; k < NY; k++)
#pragma unroll
            for (int j = 0; j < 2 * RQ; j++) q[k][j] = q[k][j + 1];
    }

    if (__syncthreads_or(bad ? 1 : 0) && tid == 0 && op.ctrl)
        atomicOr(&const_cast<DevCtrl *>(op.ctrl)->df_range, 1);
    if (Op::NACC > 0) {
        constexpr int NA = Op::NACC > 0 ? Op::NACC : 1;
        constexpr int W = AccWidth<TS>::value;
        __shared__ double red[NA * W * 32];
        block_reduce_store<NA>(acc, red, op.partials + blk * Op::NACC * W);
    }
}

// DFM: the FP64 march in double-float arithmetic (functors with DF set).
template <typename T, int RQ, int BY, int NY, int MINB, bool GENERIC, class Op, bool DFM = false>
__global__ void __launch_bounds__(32 * BY, MINB) stencil_kernel(Geom g, Weights<T> w, int lz, Op op) {
    constexpr int FX = 32 + 2 * RQ;
    constexpr int FY = BY * NY + 2 * RQ;
    __shared__ __align__(16) T smem[2][FX * FY];
    if (op.skip()) return;
    op.init();
    const long long blk = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
    if constexpr (DFM && IsDfMarch<T>::value) {
        stencil_march_df<RQ, BY, NY, GENERIC>(g, w, lz, op, smem[0], smem[1], blockIdx.x, blockIdx.y, blockIdx.z,
                                              blk);
    } else {
        stencil_march<T, RQ, BY, NY, GENERIC>(g, w, lz, op, smem[0], smem[1], blockIdx.x, blockIdx.y,
                                              blockIdx.z, blk);
    }
}

// ---------------------------------------------------------------- two columns per lane
//
// The march above with each lane owning two adjacent columns (tile 64 x TY):
// every shared, global-load and global-store access moves a pair of values
// (8 bytes for FP32), the x neighbours of both points come from 7 paired
// shared loads (24 scalar ones otherwise) and the halo strips are staged in
// pairs, so a point costs ~6.5 shared loads instead of 15 and the halo per
// point halves.  Each point's sum is evaluated in the same order as above, so
// results are bit-identical to the one-column march.  Needs nx even and 8-byte
// aligned vectors (pairs never straddle the periodic wrap then); the functor
// provides fetch_pair / center_pair / store_pair.
template <typename T> struct Two { T a, b; };
template <typename T> struct Vec2Of;
template <> struct Vec2Of<float> { using type = float2; };
template <> struct Vec2Of<double> { using type = double2; };

template <typename T>
__device__ __forceinline__ Two<T> ld_pair(const T *p) {
    const typename Vec2Of<T>::type v = *reinterpret_cast<const typename Vec2Of<T>::type *>(p);
    return Two<T>{v.x, v.y};
}
template <typename T>
__device__ __forceinline__ void st_pair(T *p, T a, T b) {
    typename Vec2Of<T>::type v;
    v.x = a;
    v.y = b;
    *reinterpret_cast<typename Vec2Of<T>::type *>(p) = v;
}

// Two-wide arithmetic of the paired march.  FP32 uses the packed f32x2
// instructions (one instruction, two round-to-nearest results); each lane
// equals the scalar operation, so the march stays bit-identical to the
// one-column driver.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ double2 add2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 mul2(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ double2 fma2(double2 a, double2 b, double2 c) {
    return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}
template <typename P, typename T>
__device__ __forceinline__ P mk2(T a, T b) {
    P v;
    v.x = a;
    v.y = b;
    return v;
}

// Functors that set PACKED run the paired march's sums as packed f32x2
// instructions; the others (a centre operand or a reduction to keep in
// registers) keep scalar sums, which need fewer aligned register pairs.
template <class Op, class = void> struct IsPacked { static constexpr bool value = false; };
template <class Op> struct IsPacked<Op, std::void_t<decltype(Op::PACKED)>> { static constexpr bool value = Op::PACKED; };

template <typename T, int BY, int NY, class Op>
__device__ __forceinline__ void stencil_march_x2(const Geom &g, const Weights<T> &w, int lz, Op &op,
                                                 T *smem0, T *smem1, int bx, int by, int bz, long long blk) {
    constexpr int RQ = 6;
    constexpr int TX = 64;
    constexpr int TY = BY * NY;
    constexpr int FX = TX + 2 * RQ;  // even, so every pair offset is 8-byte aligned
    constexpr int NT = 32 * BY;
    constexpr int PR = TX / 2;       // pairs per top / bottom halo row (no corners: the stencil is a star)
    constexpr int HP = RQ * PR * 2 + TY * RQ;  // halo pairs: top, bottom, then RQ / 2 per side per row
    constexpr int NH = (HP + NT - 1) / NT;
    constexpr int Q = 2 * RQ + 1;
    constexpr int FY = TY + 2 * RQ;
    const unsigned long long gp = (unsigned long long)g.n - 1;  // a pair at i needs i + 1 < n
    (void)gp;

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * 32 + tx;
    const int x0 = bx * TX, y0 = by * TY;
    const int z0 = bz * lz;
    const int z1 = min(z0 + lz, g.nz);

    // The lane's columns gx, gx + 1 (gx even; partial tiles wrap to valid data).
    const bool xin = x0 + 2 * tx < g.nx;
    const int gx = wrap_index(x0 + 2 * tx, g.nx);
    int col[NY];
    bool valid[NY];
#pragma unroll
    for (int k = 0; k < NY; k++) {
        const int yy = y0 + ty * NY + k;
        col[k] = gx + wrap_index(yy, g.ny) * g.nx;
        valid[k] = xin && (yy < g.ny);
    }
    int hs[NH], ho[NH];
#pragma unroll
    for (int s = 0; s < NH; s++) {
        const int h = tid + s * NT;
        hs[s] = -1;
        ho[s] = 0;
        if (h < HP) {
            int fy, fx;
            if (h < RQ * PR) {                      // top strip
                fy = h / PR; fx = RQ + 2 * (h % PR);
            } else if (h < 2 * RQ * PR) {           // bottom strip
                const int hh = h - RQ * PR;
                fy = RQ + TY + hh / PR; fx = RQ + 2 * (hh % PR);
            } else {                                // left / right strips
                const int hh = h - 2 * RQ * PR;
                const int row = hh / RQ, c = hh % RQ;
                fy = RQ + row;
                fx = c < RQ / 2 ? 2 * c : TX + 2 * c;
            }
            hs[s] = fy * FX + fx;
            ho[s] = wrap_index(x0 - RQ + fx, g.nx) + wrap_index(y0 - RQ + fy, g.ny) * g.nx;
        }
    }

    Acc<T> acc[Op::NACC > 0 ? Op::NACC : 1];
#pragma unroll
    for (int a = 0; a < (Op::NACC > 0 ? Op::NACC : 1); a++) acc[a].zero();

    using PT = typename Vec2Of<T>::type;
    constexpr bool PACK = IsPacked<Op>::value;
    PT q[NY][Q];  // the z ring of both columns, as register pairs
    unsigned zl = (unsigned)wrap_index(z0 - RQ, g.nz);
    const unsigned nxy = (unsigned)g.nxy, nz = (unsigned)g.nz;
#pragma unroll
    for (int s = 0; s < 2 * RQ; s++) {
        const unsigned base = zl * nxy;
#pragma unroll
        for (int k = 0; k < NY; k++) {
            const Two<T> v = op.fetch_pair(LSG_IX(base + col[k], gp));
            q[k][s] = mk2<PT>(v.a, v.b);
        }
        zl = (zl + 1 == nz) ? 0u : zl + 1;
    }

    Two<T> qn[NY], hn[NH], cn[NY];
    {
        const unsigned lb = zl * nxy, zb = (unsigned)z0 * nxy;
#pragma unroll
        for (int k = 0; k < NY; k++) {
            qn[k] = op.fetch_pair(LSG_IX(lb + col[k], gp));
            cn[k] = op.center_pair(LSG_IX(zb + col[k], gp));
        }
#pragma unroll
        for (int s = 0; s < NH; s++)
            if (hs[s] >= 0) hn[s] = op.fetch_pair(LSG_IX(zb + ho[s], gp));
        zl = (zl + 1 == nz) ? 0u : zl + 1;
    }

    T *sm = smem0;
    int z = z0;
    auto step = [&](auto phase) -> bool {
        constexpr int P = decltype(phase)::value;
        constexpr int HEAD = (P + Q - 1) % Q;
        constexpr int CEN = (P + RQ) % Q;
        const unsigned zbase = (unsigned)z * nxy;
#pragma unroll
        for (int k = 0; k < NY; k++) {
            q[k][HEAD] = mk2<PT>(qn[k].a, qn[k].b);
            *reinterpret_cast<PT *>(sm + LSG_IX((RQ + ty * NY + k) * FX + RQ + 2 * tx, FX * FY - 1)) = q[k][CEN];
        }
#pragma unroll
        for (int s = 0; s < NH; s++)
            if (hs[s] >= 0) st_pair(sm + LSG_IX(hs[s], FX * FY - 1), hn[s].a, hn[s].b);
        Two<T> cc[NY];
#pragma unroll
        for (int k = 0; k < NY; k++) cc[k] = cn[k];
        if (z + 1 < z1) {
            const unsigned lb = zl * nxy, nb = zbase + nxy;
#pragma unroll
            for (int k = 0; k < NY; k++) {
                qn[k] = op.fetch_pair(LSG_IX(lb + col[k], gp));
                cn[k] = op.center_pair(LSG_IX(nb + col[k], gp));
            }
#pragma unroll
            for (int s = 0; s < NH; s++)
                if (hs[s] >= 0) hn[s] = op.fetch_pair(LSG_IX(nb + ho[s], gp));
            zl = (zl + 1 == nz) ? 0u : zl + 1;
        }
        __syncthreads();
        const T *col0 = sm + (RQ + ty * NY) * FX + RQ + 2 * tx;
        // y neighbours of both columns for rows r0-RQ .. r0+NY-1+RQ (own rows from the queue)
        PT yv[NY + 2 * RQ];
#pragma unroll
        for (int j = 0; j < RQ; j++) {
            yv[j] = *reinterpret_cast<const PT *>(col0 + (j - RQ) * FX);
            yv[RQ + NY + j] = *reinterpret_cast<const PT *>(col0 + (NY + j) * FX);
        }
#pragma unroll
        for (int k = 0; k < NY; k++) yv[RQ + k] = q[k][CEN];
#pragma unroll
        for (int k = 0; k < NY; k++) {
            // x window: columns gx-RQ .. gx+1+RQ of row k as RQ+1 pairs; pair j
            // holds columns gx-RQ+2j and gx-RQ+2j+1
            PT xp[RQ + 1];
#pragma unroll
            for (int j = 0; j <= RQ; j++) xp[j] = *reinterpret_cast<const PT *>(col0 + k * FX - RQ + 2 * j);
            PT acc2;
            if constexpr (PACK) {  // packed two-wide arithmetic
                acc2 = mul2(mk2<PT>(w.w[0], w.w[0]), q[k][CEN]);
#pragma unroll
                for (int p = 1; p <= RQ; p++) {
                    // x pair at distance p: (col gx-p + col gx+p, col gx+1-p + col gx+1+p)
                    PT xs;
                    if ((RQ - p) % 2 == 0)  // both operands are loaded pairs
                        xs = add2(xp[(RQ - p) / 2], xp[(RQ + p) / 2]);
                    else
                        xs = mk2<PT>(xp[(RQ - p) / 2].y + xp[(RQ + p) / 2].y,
                                     xp[(RQ + 1 - p) / 2].x + xp[(RQ + 1 + p) / 2].x);
                    const PT ys = add2(yv[RQ + k - p], yv[RQ + k + p]);
                    const PT zs = add2(q[k][(CEN + Q - p) % Q], q[k][(CEN + p) % Q]);
                    acc2 = fma2(mk2<PT>(w.w[p], w.w[p]), add2(add2(xs, ys), zs), acc2);
                }
            } else {  // the same sums, one column at a time
                T aa = w.w[0] * q[k][CEN].x, ab = w.w[0] * q[k][CEN].y;
#pragma unroll
                for (int p = 1; p <= RQ; p++) {
                    const T xm_a = ((RQ - p) % 2 == 0) ? xp[(RQ - p) / 2].x : xp[(RQ - p) / 2].y;
                    const T xp_a = ((RQ + p) % 2 == 0) ? xp[(RQ + p) / 2].x : xp[(RQ + p) / 2].y;
                    const T xm_b = ((RQ + 1 - p) % 2 == 0) ? xp[(RQ + 1 - p) / 2].x : xp[(RQ + 1 - p) / 2].y;
                    const T xp_b = ((RQ + 1 + p) % 2 == 0) ? xp[(RQ + 1 + p) / 2].x : xp[(RQ + 1 + p) / 2].y;
                    const T sa = (xm_a + xp_a) + (yv[RQ + k - p].x + yv[RQ + k + p].x);
                    const T sb = (xm_b + xp_b) + (yv[RQ + k - p].y + yv[RQ + k + p].y);
                    const T za = q[k][(CEN + Q - p) % Q].x + q[k][(CEN + p) % Q].x;
                    const T zb = q[k][(CEN + Q - p) % Q].y + q[k][(CEN + p) % Q].y;
                    aa = fma(w.w[p], sa + za, aa);
                    ab = fma(w.w[p], sb + zb, ab);
                }
                acc2 = mk2<PT>(aa, ab);
            }
            if (valid[k] && LSG_IX_OK(zbase + col[k], gp))
                op.store_pair(zbase + col[k], Two<T>{q[k][CEN].x, q[k][CEN].y}, Two<T>{acc2.x, acc2.y}, cc[k], acc);
        }
        sm = (sm == smem0) ? smem1 : smem0;
        return ++z < z1;
    };
    while (z < z1) {
        if (!unrolled_steps<0, Q>(step)) break;
    }

    if (Op::NACC > 0) {
        constexpr int NA = Op::NACC > 0 ? Op::NACC : 1;
        constexpr int W = AccWidth<T>::value;
        __shared__ double red[NA * W * 32];
        block_reduce_store<NA>(acc, red, op.partials + blk * Op::NACC * W);
    }
}

template <typename T, int BY, int NY, int MINB, class Op>
__global__ void __launch_bounds__(32 * BY, MINB) stencil_x2_kernel(Geom g, Weights<T> w, int lz, Op op) {
    constexpr int FX = 64 + 12;
    constexpr int FY = BY * NY + 12;
    __shared__ __align__(16) T smem[2][FX * FY];
    if (op.skip()) return;
    op.init();
    const long long blk = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
    stencil_march_x2<T, BY, NY>(g, w, lz, op, smem[0], smem[1], blockIdx.x, blockIdx.y, blockIdx.z, blk);
}

}  // namespace lsg
