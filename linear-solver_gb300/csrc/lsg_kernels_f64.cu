// FP64 instantiation of the solver kernels, plus the FP64 pieces of the
// mixed-precision solver.
#include "lsg_kernels.cuh"

namespace lsg {

template struct Kernels<double>;
template cudaError_t ir_residual<double, float>(const StencilLaunch &, const Weights<double> &,
                                                const double *, const double *, float *, double *,
                                                const DevCtrl *, int);
template cudaError_t ir_correct<double, float>(double *, float *, long long, cudaStream_t);
template cudaError_t rhs_mean<double>(const double *, long long, double *, DevCtrl *, cudaStream_t);
template cudaError_t deflate_x<double>(double *, long long, double *, DevCtrl *, double, double, cudaStream_t);

template cudaError_t ir_residual_const<double, float>(const double *, float *, long long, double *, int,
                                                     const DevCtrl *, double, double, cudaStream_t);
template cudaError_t zero_check<double>(const double *, long long, DevCtrl *, cudaStream_t);

}  // namespace lsg
