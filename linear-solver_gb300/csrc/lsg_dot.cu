// lsg_dot.cu — batched inner products that stay on the device:
//   out[k] = sum_i conj(x_k[i]) y_k[i]   (real vectors: sum_i x_k[i] y_k[i])
// for `count` vectors of n values stored back to back, accumulated like the
// solvers' reductions (FP64, or double-float for FP32 / complex64 vectors),
// in fixed order (per-block partials, then one block per vector), with no host
// synchronisation.  The autograd binding uses it for dL/dsigma = -x^H lambda.
#include <cuda_runtime.h>

#include <algorithm>

#include "lsg.h"
#include "lsg_host.h"
#include "lsg_kernels.cuh"

namespace lsg {

template <typename T>
__global__ void __launch_bounds__(kReduceThreads) dot_partials_kernel(const T *__restrict__ x,
                                                                      const T *__restrict__ y, long long n,
                                                                      double *part) {
    constexpr int W = AccWidth<T>::value;
    __shared__ double red[W * 32];
    const long long k = blockIdx.y;
    const T *xk = x + k * n, *yk = y + k * n;
    Acc<T> acc[1];
    acc[0].zero();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        acc[0].add_prod(ldg(xk + i), ldg(yk + i));
    block_reduce_store<1>(acc, red, part + (k * gridDim.x + blockIdx.x) * W);
}

// One block per vector: component c of out[k] = sum over the nblk partials.
__global__ void __launch_bounds__(kReduceThreads) dot_finalize_kernel(const double *part, int nblk, int w,
                                                                      double *out) {
    __shared__ double red[kReduceThreads / 32];
    const long long k = blockIdx.x;
    for (int c = 0; c < w; c++) {
        double s = 0.0;
        for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += part[(k * nblk + b) * w + c];
        s = warp_sum(s);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
            t = warp_sum(t);
            if (threadIdx.x == 0) out[k * w + c] = t;
        }
        __syncthreads();
    }
}

template <typename T>
static int dot_t(int count, long long n, const void *x, const void *y, double *out, double *scratch,
                 cudaStream_t s) {
    constexpr int W = AccWidth<T>::value;
    const int nblk = lsg_dot_blocks(n);
    dim3 grid((unsigned)nblk, (unsigned)count);
    dot_partials_kernel<T><<<grid, kReduceThreads, 0, s>>>((const T *)x, (const T *)y, n, scratch);
    dot_finalize_kernel<<<count, kReduceThreads, 0, s>>>(scratch, nblk, W, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(LSG_CUDA_ERROR, "lsg_dot: %s", cudaGetErrorString(e));
    return LSG_OK;
}

}  // namespace lsg

extern "C" {

int lsg_dot_blocks(long long n) {
    const long long need = (n + lsg::kReduceThreads - 1) / lsg::kReduceThreads;
    return (int)std::max<long long>(1, std::min<long long>(need, (long long)lsg::sm_count() * 2));
}

int lsg_dot(int dtype, int count, long long n, const void *d_x, const void *d_y, double *d_out,
            double *d_scratch, void *stream) {
    using namespace lsg;
    if (count < 1 || count > 65535 || n < 1) return set_error(LSG_BAD_ARG, "lsg_dot: count %d, n %lld", count, n);
    if (!d_x || !d_y || !d_out || !d_scratch) return set_error(LSG_BAD_ARG, "lsg_dot: NULL pointer");
    cudaStream_t s = (cudaStream_t)stream;
    switch (dtype) {
    case LSG_F64: return dot_t<double>(count, n, d_x, d_y, d_out, d_scratch, s);
    case LSG_F32: return dot_t<float>(count, n, d_x, d_y, d_out, d_scratch, s);
    case LSG_C128: return dot_t<cplx<double>>(count, n, d_x, d_y, d_out, d_scratch, s);
    case LSG_C64: return dot_t<cplx<float>>(count, n, d_x, d_y, d_out, d_scratch, s);
    default: return set_error(LSG_BAD_ARG, "lsg_dot: unknown dtype %d", dtype);
    }
}

}  // extern "C"
