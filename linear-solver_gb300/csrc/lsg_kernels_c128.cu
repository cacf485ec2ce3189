// complex128 instantiation of the AAR kernels (shifted Helmholtz), plus the
// complex128 pieces of the mixed-precision solver.
#include "lsg_kernels.cuh"

namespace lsg {

template struct Kernels<cplx<double>>;
template cudaError_t ir_residual<cplx<double>, cplx<float>>(const StencilLaunch &,
                                                            const Weights<cplx<double>> &,
                                                            const cplx<double> *,
                                                            const cplx<double> *, cplx<float> *,
                                                            double *, const DevCtrl *, int);
template cudaError_t ir_correct<cplx<double>, cplx<float>>(cplx<double> *, cplx<float> *, long long,
                                                           cudaStream_t);
template cudaError_t rhs_mean<cplx<double>>(const cplx<double> *, long long, double *, DevCtrl *, cudaStream_t);
template cudaError_t deflate_x<cplx<double>>(cplx<double> *, long long, double *, DevCtrl *, double, double,
                                             cudaStream_t);

template cudaError_t ir_residual_const<cplx<double>, cplx<float>>(const cplx<double> *, cplx<float> *, long long, double *, int,
                                                     const DevCtrl *, double, double, cudaStream_t);
template cudaError_t zero_check<cplx<double>>(const cplx<double> *, long long, DevCtrl *, cudaStream_t);

}  // namespace lsg
