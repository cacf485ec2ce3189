// complex64 instantiation of the AAR kernels (the inner solver of the
// mixed-precision shifted-Helmholtz AAR).
#include "lsg_kernels.cuh"

namespace lsg {

template struct Kernels<cplx<float>>;

}  // namespace lsg
