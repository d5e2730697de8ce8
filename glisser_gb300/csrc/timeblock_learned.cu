// Learned-starter instantiations of the single-system time-block kernel,
// with the float-float or the FP64 kick (the network is compiled in only
// here, so the plain kernels keep their register allocation).  Specialised
// for one and four planets besides the Sun; other counts use the generic
// planet loop.
#include "timeblock_kernel.cuh"

namespace glisser {

cudaError_t launch_timeblock_learned(const tile::Common& p, const glisser_planet_block* pl, uint32_t n, size_t smem,
                                     cudaStream_t stream)
{
    return p.kick64 ? launch_variant<true, true>(p, pl, n, smem, stream)
                    : launch_variant<true, false>(p, pl, n, smem, stream);
}

}  // namespace glisser
