// Learned-starter instantiations of the ensemble kernel, float-float kick.
#include "batched_kernel.cuh"

namespace glisser {

GLISSER_BATCHED_VARIANT_LAUNCH(launch_batched_learned)
{
    return launch_batched_variant<true, false>(p, sys, items, n_items, queue, npl, shape, smem, stream);
}

}  // namespace glisser
