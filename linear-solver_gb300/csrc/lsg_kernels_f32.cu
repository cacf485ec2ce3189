// FP32 instantiation of the solver kernels (vectors, history and stencil in
// FP32; reductions in double-float, converted to FP64 per block).
#include "lsg_kernels.cuh"

namespace lsg {

template struct Kernels<float>;

}  // namespace lsg
