// Learned-starter instantiations of the single-system time-block kernel
// (the MLP guess is compiled in only here, so the plain kernels keep their
// register allocation).  Specialised for one and four planets besides the
// Sun; other counts use the generic planet loop.
#include "timeblock_kernel.cuh"

namespace glisser {

cudaError_t launch_timeblock_learned(const tile::Common& p, const glisser_planet_block* pl, uint32_t n, size_t smem,
                                     cudaStream_t stream)
{
    switch (pl->npl - 1) {
    case 1: return launch_np<1, true>(p, pl, n, smem, stream);
    case 4: return launch_np<4, true>(p, pl, n, smem, stream);
    default: return launch_np<0, true>(p, pl, n, smem, stream);
    }
}

}  // namespace glisser
