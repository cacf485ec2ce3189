// lsg_accum.cuh — per-thread accumulators with FP64-class precision.
//
// FP64 on this part runs at about 1/70 of the FP32 rate, so sums of FP32
// products are kept as unevaluated float pairs (hi + lo, "double-float"):
// each product is formed exactly (p = a*b, e = fma(a, b, -p)) and added to
// hi with Knuth's two-sum, the rounding errors collecting in lo.  That gives
// the FP64-accumulation accuracy the FP32 solver needs while issuing only
// FP32 instructions; the pair is converted to a double once per thread, at
// the block reduction.  FP64 vectors accumulate in plain doubles.
#pragma once

namespace lsg {

template <typename T>
struct Acc;

template <>
struct Acc<double> {
    double v;
    __device__ __forceinline__ void zero() { v = 0.0; }
    __device__ __forceinline__ void add(double a) { v += a; }
    __device__ __forceinline__ void add_prod(double a, double b) { v = fma(a, b, v); }
    __device__ __forceinline__ double get() const { return v; }
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

template <>
struct Acc<float> {
    float hi, lo;
    __device__ __forceinline__ void zero() { hi = 0.f; lo = 0.f; }
    __device__ __forceinline__ void add(float a) {
        float s, e;
        two_sum(hi, a, s, e);
        hi = s;
        lo += e;
    }
    __device__ __forceinline__ void add_prod(float a, float b) {
        const float p = a * b;
        const float pe = fmaf(a, b, -p);
        float s, e;
        two_sum(hi, p, s, e);
        hi = s;
        lo += e + pe;
    }
    __device__ __forceinline__ double get() const { return (double)hi + (double)lo; }
};

// Warp-wide sum of double-float pairs (FP32 instructions only).
__device__ __forceinline__ void df_warp_sum(float &hi, float &lo) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
        float s, e;
        two_sum(hi, h2, s, e);
        hi = s;
        lo += l2 + e;
    }
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sums NV per-thread accumulators over the block and writes the NV totals
// (FP64) to out[0..NV).  `scratch` is NV * 32 doubles of shared memory.
// FP32 accumulators are reduced as double-float pairs with FP32 instructions;
// only the NV final conversions to double touch the (slow) FP64 pipe.
// perm (optional, shared memory): total k goes to out[perm[k]].  s1, s2:
// powers of two the (double) totals are multiplied by, one after the other
// (scaled double-float sums).
template <int NV, typename T>
__device__ __forceinline__ void block_reduce_store(Acc<T> (&acc)[NV], double *scratch, double *out,
                                                   const int *perm = nullptr, double s1 = 1.0, double s2 = 1.0) {
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = tid & 31, warp = tid >> 5;
    const int nwarps = (blockDim.x * blockDim.y) >> 5;
    if constexpr (sizeof(T) == 8) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            const double s = warp_sum_d(acc[k].get());
            if (lane == 0) scratch[k * nwarps + warp] = s;
        }
        __syncthreads();
        for (int k = warp; k < NV; k += nwarps) {
            double s = lane < nwarps ? scratch[k * nwarps + lane] : 0.0;
            s = warp_sum_d(s);
            if (lane == 0) out[perm ? perm[k] : k] = s;
        }
    } else {
        float2 *sf = reinterpret_cast<float2 *>(scratch);
#pragma unroll
        for (int k = 0; k < NV; k++) {
            float hi = acc[k].hi, lo = acc[k].lo;
            df_warp_sum(hi, lo);
            if (lane == 0) sf[k * nwarps + warp] = make_float2(hi, lo);
        }
        __syncthreads();
        for (int k = warp; k < NV; k += nwarps) {
            float hi = 0.f, lo = 0.f;
            if (lane < nwarps) { const float2 v = sf[k * nwarps + lane]; hi = v.x; lo = v.y; }
            df_warp_sum(hi, lo);
            if (lane == 0) out[perm ? perm[k] : k] = ((double)hi + (double)lo) * s1 * s2;
        }
    }
}

}  // namespace lsg
