// Batched kernels for cplx<double> vectors.
#include "lsg_batch.cuh"

namespace lsg {
template struct BatchKernels<cplx<double>>;
}  // namespace lsg
