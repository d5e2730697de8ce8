// Single-system time-block kernel template, included by the translation
// units that instantiate it (plain starters in timeblock.cu, the learned
// starter in timeblock_learned.cu; disjoint instantiations, internal linkage).
#pragma once
#include "tile.cuh"

namespace glisser {
namespace {

using namespace tile;

// CTAs per SM the register allocation is sized for.  Once the drift's
// reciprocal square root and small-step Stumpff tier moved most of their
// FP64 work to the FP32 and integer pipes, the kernel became latency-bound
// with neither pipe saturated, and resident warps count: 16 CTAs of 64
// threads (64 registers, a few dozen bytes of spills; 32-step planet-log
// chunks, so that shared memory admits 16 with four planets) measured 7 %
// faster than 10 CTAs at 80 registers on the plain-giants workload and 2.5 %
// on the scattered disk; 18 and 20 CTAs spill more.
#ifndef GLISSER_TB_MIN_BLOCKS
#define GLISSER_TB_MIN_BLOCKS 16
#endif

// The learned-starter kernel runs the network per lane, inline, only where
// the series starter is outside its domain.  Its register allocation follows
// the plain kernel's occupancy (16 CTAs of 64 per SM: 64 registers), so that
// the network costs no occupancy on the steps that do not run it: at 80
// registers (12 CTAs) it ran 0.991x the plain kernel on the scattered disk,
// where 0.1 % of drifts take the network, and 1.062x on the close-eccentric
// workload, where every drift does; at 64 registers 1.016x and 1.071x (the
// spills sit around the network).  The network's shape
// (mlp_forward: four rows of the hidden layer per pass, two activation
// reads in flight) was chosen for a register budget.
#ifndef GLISSER_TB_MIN_BLOCKS_LEARNED
#define GLISSER_TB_MIN_BLOCKS_LEARNED 16
#endif
constexpr int TB_NET_ROWS = 4;
constexpr int TB_NET_QU = 2;

// Particles per thread of the plain-starter kernel (a build-time tuning
// knob; the learned kernel keeps one).  Two (118 registers, 8 CTAs per SM)
// measured 14 % slower on the plain-giants workload and 36 % on the
// scattered disk, where the warp-uniform Stumpff tiers diverge more often.
#ifndef GLISSER_TB_PPT
#define GLISSER_TB_PPT 1
#endif

template <int NP, bool LEARNED, bool KICK64>
__global__ void __launch_bounds__(BLOCK_THREADS, LEARNED ? GLISSER_TB_MIN_BLOCKS_LEARNED : GLISSER_TB_MIN_BLOCKS)
    timeblock_kernel(const Common p, const double* log, const double* m, const double* rh, const uint32_t* pid,
                     uint32_t n)
{
    extern __shared__ __align__(128) double stage[];
    __shared__ CtaShared sh;
    load_planet_constants(sh, p.npl, m, rh, pid);
    init_barriers(sh);
    __syncthreads();
    uint32_t phase[2] = { 0, 0 };
    constexpr int PPT = LEARNED ? 1 : GLISSER_TB_PPT;
    const uint32_t first = blockIdx.x * (uint32_t)(BLOCK_THREADS * PPT);
    run_tile<NP, BLOCK_THREADS, PPT, LEARNED, KICK64, TB_NET_ROWS, TB_NET_QU>(
        p, log, first, min((uint32_t)(BLOCK_THREADS * PPT), n - first), stage, sh, phase);
}

template <int NP, bool LEARNED, bool KICK64>
cudaError_t launch_np(const Common& p, const glisser_planet_block* pl, uint32_t n, size_t smem, cudaStream_t stream)
{
    auto kern = timeblock_kernel<NP, LEARNED, KICK64>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const uint32_t per_cta = (uint32_t)BLOCK_THREADS * (LEARNED ? 1u : (uint32_t)GLISSER_TB_PPT);
    const uint32_t grid = (n + per_cta - 1) / per_cta;
    kern<<<grid, BLOCK_THREADS, smem, stream>>>(p, pl->log, pl->m, pl->rh, pl->id, n);
    return cudaGetLastError();
}

// Dispatch over the planet count for one kernel variant.
template <bool LEARNED, bool KICK64>
cudaError_t launch_variant(const Common& p, const glisser_planet_block* pl, uint32_t n, size_t smem,
                           cudaStream_t stream)
{
    if constexpr (LEARNED) {
        // learned instantiations: one and four planets besides the Sun
        // specialised, other counts on the generic planet loop
        switch (pl->npl - 1) {
        case 1: return launch_np<1, true, KICK64>(p, pl, n, smem, stream);
        case 4: return launch_np<4, true, KICK64>(p, pl, n, smem, stream);
        default: return launch_np<0, true, KICK64>(p, pl, n, smem, stream);
        }
    } else {
        switch (pl->npl - 1) {
        case 1: return launch_np<1, false, KICK64>(p, pl, n, smem, stream);
        case 2: return launch_np<2, false, KICK64>(p, pl, n, smem, stream);
        case 3: return launch_np<3, false, KICK64>(p, pl, n, smem, stream);
        case 4: return launch_np<4, false, KICK64>(p, pl, n, smem, stream);
        case 5: return launch_np<5, false, KICK64>(p, pl, n, smem, stream);
        case 6: return launch_np<6, false, KICK64>(p, pl, n, smem, stream);
        case 7: return launch_np<7, false, KICK64>(p, pl, n, smem, stream);
        case 8: return launch_np<8, false, KICK64>(p, pl, n, smem, stream);
        default: return launch_np<0, false, KICK64>(p, pl, n, smem, stream);
        }
    }
}

}  // namespace

// Launches of the variants compiled in other translation units (each unit
// instantiates one variant, so that the units compile in parallel and keep
// their register allocations apart): plain starters with the FP64 kick
// (timeblock_kick64.cu), the learned starter with either kick
// (timeblock_learned.cu).
cudaError_t launch_timeblock_kick64(const tile::Common& p, const glisser_planet_block* pl, uint32_t n, size_t smem,
                                    cudaStream_t stream);
cudaError_t launch_timeblock_learned(const tile::Common& p, const glisser_planet_block* pl, uint32_t n, size_t smem,
                                     cudaStream_t stream);

}  // namespace glisser
