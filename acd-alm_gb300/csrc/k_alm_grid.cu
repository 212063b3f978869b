// Compiles the ALM solve of one LP on the whole GPU (grid team), fused multiply-adds.
#include "kernels.cuh"

namespace acd {

const void * kernel_alm_grid_fast() { return (const void *)alm_kernel<false>; }

}  // namespace acd
