// Single-system time-block kernel template, included by the translation
// units that instantiate it (plain starters in timeblock.cu, the learned
// starter in timeblock_learned.cu; disjoint instantiations, internal linkage).
#pragma once
#include "tile.cuh"

namespace glisser {
namespace {

using namespace tile;

// CTAs per SM the register allocation is sized for.  With the planet kick
// and the starter in float-float on the FP32 pipe, longer dependency chains
// make resident warps count: 10 CTAs of 64 threads (with 64-step planet-log
// chunks, so that shared memory admits them) measured 1 % faster than 8 and
// 12, and 4 % faster than the 7 that 128-step chunks allow.
#ifndef GLISSER_TB_MIN_BLOCKS
#define GLISSER_TB_MIN_BLOCKS 10
#endif

// The learned-starter kernel carries the MLP's 32 hidden activations on top
// of the drift's registers.  A bound of 7 CTAs per SM (ptxas still picks 128
// registers, spilling 96 bytes) measured 1.6 % faster than 8 (128, 136
// bytes spilled) and 8 % faster than 6 or 9.
#ifndef GLISSER_TB_MIN_BLOCKS_LEARNED
#define GLISSER_TB_MIN_BLOCKS_LEARNED 7
#endif

template <int NP, bool LEARNED>
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
    const uint32_t first = blockIdx.x * BLOCK_THREADS;
    run_tile<NP, BLOCK_THREADS, 1, LEARNED>(p, log, first, min((uint32_t)BLOCK_THREADS, n - first), stage, sh, phase);
}

template <int NP, bool LEARNED>
cudaError_t launch_np(const Common& p, const glisser_planet_block* pl, uint32_t n, size_t smem, cudaStream_t stream)
{
    auto kern = timeblock_kernel<NP, LEARNED>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    uint32_t grid = (n + BLOCK_THREADS - 1) / BLOCK_THREADS;
    kern<<<grid, BLOCK_THREADS, smem, stream>>>(p, pl->log, pl->m, pl->rh, pl->id, n);
    return cudaGetLastError();
}

}  // namespace

// Learned-starter launch (timeblock_learned.cu).
cudaError_t launch_timeblock_learned(const tile::Common& p, const glisser_planet_block* pl, uint32_t n, size_t smem,
                                     cudaStream_t stream);

}  // namespace glisser
