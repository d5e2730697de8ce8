// Learned-starter instantiations of the ensemble kernel (four planets
// besides the Sun specialised, other counts on the generic planet loop).
#include "batched_kernel.cuh"

namespace glisser {

cudaError_t launch_batched_learned(const tile::Common& p, const BatchSystems& sys, const BatchItem* items,
                                   const uint32_t* n_items, uint32_t* queue, uint32_t npl, const BatchShape& shape,
                                   size_t smem, cudaStream_t stream)
{
    return npl == 5 ? launch_batched_np<4, true>(p, sys, items, n_items, queue, shape, smem, stream)
                    : launch_batched_np<0, true>(p, sys, items, n_items, queue, shape, smem, stream);
}

}  // namespace glisser
