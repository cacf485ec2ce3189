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

}  // namespace lsg
