// Compiles the ALM solve of one LP on the whole GPU (grid team), the reference's
// separate rounding of products and sums.
#include "kernels.cuh"

namespace acd {

const void * kernel_alm_grid_exact() { return (const void *)alm_kernel<true>; }

}  // namespace acd
