// Compiles approx_solve and mpg_solve on the whole GPU (grid team).
#include "kernels.cuh"

namespace acd {

const void * kernel_approx_grid(bool exact)
{
        return exact ? (const void *)approx_kernel<true> : (const void *)approx_kernel<false>;
}

const void * kernel_mpg_grid() { return (const void *)mpg_kernel<false>; }

}  // namespace acd
