// Batched kernels for double vectors.
#include "lsg_batch.cuh"

namespace lsg {
template struct BatchKernels<double>;
}  // namespace lsg
