// Plain-starter instantiations of the single-system time-block kernel with
// the planet kick and its radius tests in FP64 (GLISSER_KICK_FP64), the
// reference's arithmetic for that part of the step (src/wh.cu:142-172).
#include "timeblock_kernel.cuh"

namespace glisser {

cudaError_t launch_timeblock_kick64(const tile::Common& p, const glisser_planet_block* pl, uint32_t n, size_t smem,
                                    cudaStream_t stream)
{
    return launch_variant<false, true>(p, pl, n, smem, stream);
}

}  // namespace glisser
