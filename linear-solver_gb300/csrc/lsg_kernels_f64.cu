// FP64 instantiation of the solver kernels, plus the FP64 pieces of the
// mixed-precision refinement loop.
#include "lsg_kernels.cuh"

namespace lsg {

template struct Kernels<double>;

cudaError_t ir_residual(const StencilLaunch &L, const Weights<double> &w, const double *x,
                        const double *b, float *r32, double *partials, const DevCtrl *ctrl) {
    IrResidualOp op{x, b, r32, partials, ctrl};
    return launch_stencil<double>(L, w, op);
}

// x64 += e32; e32 = 0 (the correction is folded into x and restarts at zero).
__global__ void ir_correct_kernel(double *__restrict__ x, float *__restrict__ e, long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        x[i] += (double)e[i];
        e[i] = 0.0f;
    }
}

cudaError_t ir_correct(double *x, float *e, long long n, cudaStream_t s) {
    const int blocks = (int)std::min<long long>((n + kReduceThreads - 1) / kReduceThreads, 152 * 8);
    ir_correct_kernel<<<blocks, kReduceThreads, 0, s>>>(x, e, n);
    return cudaGetLastError();
}

}  // namespace lsg
