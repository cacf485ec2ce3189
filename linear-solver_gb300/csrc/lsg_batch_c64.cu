// Batched kernels for cplx<float> vectors.
#include "lsg_batch.cuh"

namespace lsg {
template struct BatchKernels<cplx<float>>;
}  // namespace lsg
