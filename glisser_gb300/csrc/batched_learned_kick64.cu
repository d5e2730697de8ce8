// Learned-starter instantiations of the ensemble kernel with the planet kick
// and its radius tests in FP64 (GLISSER_KICK_FP64).
#include "batched_kernel.cuh"

namespace glisser {

GLISSER_BATCHED_VARIANT_LAUNCH(launch_batched_learned_kick64)
{
    return launch_batched_variant<true, true>(p, sys, items, n_items, queue, npl, shape, smem, stream);
}

}  // namespace glisser
