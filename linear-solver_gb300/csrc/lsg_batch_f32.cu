// Batched kernels for float vectors.
#include "lsg_batch.cuh"

namespace lsg {
template struct BatchKernels<float>;
}  // namespace lsg
