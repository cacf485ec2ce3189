// lsg_complex.cuh — complex scalars for the shifted-Helmholtz solvers.
//
// cplx<R> is an 8- or 16-byte (re, im) pair with the arithmetic the solver
// kernels use, so the stencil driver, the Richardson / residual functors and
// the Anderson update instantiate for complex vectors unchanged.  The FD
// weights stay real except the centre weight 3 a c_0 + sigma, which carries
// the complex shift; the Jacobi factor 1 / (3 a c_0 + sigma) is complex too.
#pragma once

#include <cuda_runtime.h>

#include "lsg_accum.cuh"

namespace lsg {

template <typename R>
struct alignas(2 * sizeof(R)) cplx {
    R x, y;
    cplx() = default;
    __host__ __device__ constexpr cplx(R re, R im = R(0)) : x(re), y(im) {}
    template <typename S>
    __host__ __device__ explicit cplx(const cplx<S> &o) : x((R)o.x), y((R)o.y) {}
};

// The real fma overloads stay visible next to the complex ones below.
using ::fma;

template <typename T> struct RealOf { using type = T; };
template <typename R> struct RealOf<cplx<R>> { using type = R; };
template <typename T> struct IsCplx { static constexpr bool value = false; };
template <typename R> struct IsCplx<cplx<R>> { static constexpr bool value = true; };

template <typename R>
__host__ __device__ __forceinline__ cplx<R> operator+(cplx<R> a, cplx<R> b) { return cplx<R>(a.x + b.x, a.y + b.y); }
template <typename R>
__host__ __device__ __forceinline__ cplx<R> operator-(cplx<R> a, cplx<R> b) { return cplx<R>(a.x - b.x, a.y - b.y); }
template <typename R>
__host__ __device__ __forceinline__ cplx<R> operator-(cplx<R> a) { return cplx<R>(-a.x, -a.y); }
template <typename R>
__host__ __device__ __forceinline__ cplx<R> operator*(cplx<R> a, cplx<R> b) {
    return cplx<R>(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
template <typename R>
__host__ __device__ __forceinline__ cplx<R> operator*(R s, cplx<R> a) { return cplx<R>(s * a.x, s * a.y); }
template <typename R>
__host__ __device__ __forceinline__ cplx<R> &operator+=(cplx<R> &a, cplx<R> b) { a = a + b; return a; }
template <typename R>
__host__ __device__ __forceinline__ cplx<R> conj(cplx<R> a) { return cplx<R>(a.x, -a.y); }
// a * b + c
template <typename R>
__host__ __device__ __forceinline__ cplx<R> fma(cplx<R> a, cplx<R> b, cplx<R> c) {
    return cplx<R>(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
template <typename R>
__host__ __device__ __forceinline__ cplx<R> fma(R a, cplx<R> b, cplx<R> c) {
    return cplx<R>(fma(a, b.x, c.x), fma(a, b.y, c.y));
}

template <typename R>
__device__ __forceinline__ cplx<R> ldg(const cplx<R> *p);
template <>
__device__ __forceinline__ cplx<float> ldg(const cplx<float> *p) {
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return cplx<float>(v.x, v.y);
}
template <>
__device__ __forceinline__ cplx<double> ldg(const cplx<double> *p) {
    const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    return cplx<double>(v.x, v.y);
}

// Complex accumulator of conj(a) * b (the Hermitian inner product of
// PETSc's VecDot, PETSC_COMPLEX/AAR_Complex.c:213-216), FP64-class.
template <typename R>
struct Acc<cplx<R>> {
    Acc<R> re, im;
    __device__ __forceinline__ void zero() { re.zero(); im.zero(); }
    __device__ __forceinline__ void add_prod(cplx<R> a, cplx<R> b) {
        re.add_prod(a.x, b.x);
        re.add_prod(a.y, b.y);
        im.add_prod(a.x, b.y);
        im.add_prod(-a.y, b.x);
    }
};

// Reals per accumulator (partials layout): 1 for real, 2 for complex.
template <typename T> struct AccWidth { static constexpr int value = 1; };
template <typename R> struct AccWidth<cplx<R>> { static constexpr int value = 2; };

// Complex accumulators reduce as 2 NV real ones: out[2k] = Re, out[2k+1] = Im.
template <int NV, typename R>
__device__ __forceinline__ void block_reduce_store(Acc<cplx<R>> (&acc)[NV], double *scratch, double *out) {
    Acc<R> flat[2 * NV];
#pragma unroll
    for (int k = 0; k < NV; k++) {
        flat[2 * k] = acc[k].re;
        flat[2 * k + 1] = acc[k].im;
    }
    block_reduce_store<2 * NV, R>(flat, scratch, out);
}

}  // namespace lsg
