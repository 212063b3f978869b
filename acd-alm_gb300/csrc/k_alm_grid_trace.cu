// Compiles the ALM solve of one LP on the whole GPU (grid team) with phase
// tracing, fused multiply-adds.
#include "kernels.cuh"

namespace acd {

const void * kernel_alm_grid_trace() { return (const void *)alm_kernel<false, true>; }

}  // namespace acd
