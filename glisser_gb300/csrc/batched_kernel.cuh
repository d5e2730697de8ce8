// Ensemble (persistent work-queue) kernel template, included by the
// translation units that instantiate it (plain starters in batched.cu, the
// learned starter in batched_learned.cu; disjoint instantiations, internal
// linkage).
#pragma once
#include "tile.cuh"

namespace glisser {
namespace {

using namespace tile;

// Resident threads per SM the ensemble kernel's registers are sized for; a
// build-time tuning knob.  The plain-starter kernel is latency-bound (FP64
// pipe ~65 % busy, issue ~57 % at 5 CTAs of 128), so it is sized for 8 CTAs
// of 128 per SM (64 registers, ~100 bytes of spills; 64-step planet-log
// chunks fit 8 CTAs' shared memory): 6 % faster than 5 CTAs at 93
// registers, and ahead of 6, 7 and 9 CTAs.  The learned-starter kernel is
// sized the same: on ensembles whose every drift runs the network it
// measured 1.6 % faster at 8 CTAs (64 registers, its network's activations
// and spills in local memory) than at 4 (96 registers).
#ifndef GLISSER_BATCHED_THREADS_PER_SM
#define GLISSER_BATCHED_THREADS_PER_SM 1024
#endif
#ifndef GLISSER_BATCHED_THREADS_PER_SM_LEARNED
#define GLISSER_BATCHED_THREADS_PER_SM_LEARNED GLISSER_BATCHED_THREADS_PER_SM
#endif

// Persistent kernel over (system, tile) work items.  The learned starter
// runs its network per lane, inline, only where the series starter is
// outside its domain.
template <int NP, int CTA, int PPT, bool LEARNED, bool KICK64>
__global__ void __launch_bounds__(CTA, (LEARNED ? GLISSER_BATCHED_THREADS_PER_SM_LEARNED
                                                : GLISSER_BATCHED_THREADS_PER_SM) / CTA)
    batched_kernel(const Common p, BatchSystems sys, const BatchItem* items, const uint32_t* n_items, uint32_t* queue)
{
    extern __shared__ __align__(128) double stage[];
    __shared__ CtaShared sh;
    init_barriers(sh);
    uint32_t phase[2] = { 0, 0 };
    const uint32_t total = *n_items;
    for (;;) {
        if (threadIdx.x == 0) sh.item = atomicAdd(queue, 1u);
        __syncthreads();
        const uint32_t it = sh.item;
        if (it >= total || sh.abort) break;
        const BatchItem w = items[it];
        load_planet_constants(sh, p.npl, sys.m + (size_t)w.system * p.npl, sys.rh + (size_t)w.system * p.npl,
                              sys.id + (size_t)w.system * p.npl);
        __syncthreads();
        bool ok = run_tile<NP, CTA, PPT, LEARNED, KICK64>(p, sys.log + (size_t)w.system * sys.log_stride, w.first,
                                                          w.count, stage, sh, phase);
        __syncthreads();   // sh.item / planet constants are rewritten by the next item
        if (!ok) break;
    }
}

template <int NP, int CTA, int PPT, bool LEARNED, bool KICK64>
cudaError_t launch_batched_t(const Common& p, const BatchSystems& sys, const BatchItem* items,
                             const uint32_t* n_items, uint32_t* queue, uint32_t grid, size_t smem,
                             cudaStream_t stream)
{
    auto kern = batched_kernel<NP, CTA, PPT, LEARNED, KICK64>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (grid == 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, CTA, smem);
        grid = (uint32_t)(sms * (per > 0 ? per : 1));
    }
    kern<<<grid, CTA, smem, stream>>>(p, sys, items, n_items, queue);
    return cudaGetLastError();
}

template <int NP, bool LEARNED, bool KICK64>
cudaError_t launch_batched_np(const Common& p, const BatchSystems& sys, const BatchItem* items,
                              const uint32_t* n_items, uint32_t* queue, const BatchShape& shape, size_t smem,
                              cudaStream_t stream)
{
    const int key = shape.cta * 10 + shape.ppt;
    const uint32_t g = shape.grid;
    switch (key) {
    case 641: return launch_batched_t<NP, 64, 1, LEARNED, KICK64>(p, sys, items, n_items, queue, g, smem, stream);
    case 642: return launch_batched_t<NP, 64, 2, LEARNED, KICK64>(p, sys, items, n_items, queue, g, smem, stream);
    case 1281: return launch_batched_t<NP, 128, 1, LEARNED, KICK64>(p, sys, items, n_items, queue, g, smem, stream);
    case 1282: return launch_batched_t<NP, 128, 2, LEARNED, KICK64>(p, sys, items, n_items, queue, g, smem, stream);
    case 2561: return launch_batched_t<NP, 256, 1, LEARNED, KICK64>(p, sys, items, n_items, queue, g, smem, stream);
    case 2562: return launch_batched_t<NP, 256, 2, LEARNED, KICK64>(p, sys, items, n_items, queue, g, smem, stream);
    default: return cudaErrorInvalidValue;
    }
}

// One kernel variant: four planets besides the Sun specialised, other counts
// on the generic planet loop.
template <bool LEARNED, bool KICK64>
cudaError_t launch_batched_variant(const Common& p, const BatchSystems& sys, const BatchItem* items,
                                   const uint32_t* n_items, uint32_t* queue, uint32_t npl, const BatchShape& shape,
                                   size_t smem, cudaStream_t stream)
{
    return npl == 5 ? launch_batched_np<4, LEARNED, KICK64>(p, sys, items, n_items, queue, shape, smem, stream)
                    : launch_batched_np<0, LEARNED, KICK64>(p, sys, items, n_items, queue, shape, smem, stream);
}

}  // namespace

// Launches of the variants compiled in other translation units (one variant
// per unit): plain starters with the FP64 kick (batched_kick64.cu), the
// learned starter with the float-float kick (batched_learned.cu) and with the
// FP64 kick (batched_learned_kick64.cu).
#define GLISSER_BATCHED_VARIANT_LAUNCH(name)                                                                     \
    cudaError_t name(const tile::Common& p, const BatchSystems& sys, const BatchItem* items,                     \
                     const uint32_t* n_items, uint32_t* queue, uint32_t npl, const BatchShape& shape, size_t smem, \
                     cudaStream_t stream)
GLISSER_BATCHED_VARIANT_LAUNCH(launch_batched_kick64);
GLISSER_BATCHED_VARIANT_LAUNCH(launch_batched_learned);
GLISSER_BATCHED_VARIANT_LAUNCH(launch_batched_learned_kick64);

}  // namespace glisser
