// Ensemble time-block kernel: many independent systems (each its own
// planets and particle range) in one persistent launch.  CTAs pop
// (system, tile) items from a device work queue (one atomic per item), load
// that system's planet constants, and run the same tile routine as the
// single-system kernel, staging the item's own planet log through the bulk-
// TMA double buffer.  Items of one system are consecutive, so neighbouring
// CTAs share that system's log in L2.  The CTA size (64/128/256) and the
// particles per thread (1/2) are template parameters picked by the autotuner.
#include <cstdio>

#include "tile.cuh"

namespace glisser {

using namespace tile;

namespace {

// Persistent kernel over (system, tile) work items.
template <int NP, int CTA, int PPT>
__global__ void __launch_bounds__(CTA)
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
        bool ok = run_tile<NP, CTA, PPT>(p, sys.log + (size_t)w.system * sys.log_stride, w.first, w.count, stage, sh,
                                         phase);
        __syncthreads();   // sh.item / planet constants are rewritten by the next item
        if (!ok) break;
    }
}

}  // namespace

const char* timeblock_error();
void set_timeblock_error(const char* msg);

namespace {

template <int NP, int CTA, int PPT>
cudaError_t launch_batched_t(const Common& p, const BatchSystems& sys, const BatchItem* items,
                             const uint32_t* n_items, uint32_t* queue, uint32_t grid, size_t smem,
                             cudaStream_t stream)
{
    auto kern = batched_kernel<NP, CTA, PPT>;
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

template <int NP>
cudaError_t launch_batched_np(const Common& p, const BatchSystems& sys, const BatchItem* items,
                              const uint32_t* n_items, uint32_t* queue, const BatchShape& shape, size_t smem,
                              cudaStream_t stream)
{
    const int key = shape.cta * 10 + shape.ppt;
    switch (key) {
    case 641: return launch_batched_t<NP, 64, 1>(p, sys, items, n_items, queue, shape.grid, smem, stream);
    case 642: return launch_batched_t<NP, 64, 2>(p, sys, items, n_items, queue, shape.grid, smem, stream);
    case 1281: return launch_batched_t<NP, 128, 1>(p, sys, items, n_items, queue, shape.grid, smem, stream);
    case 1282: return launch_batched_t<NP, 128, 2>(p, sys, items, n_items, queue, shape.grid, smem, stream);
    case 2561: return launch_batched_t<NP, 256, 1>(p, sys, items, n_items, queue, shape.grid, smem, stream);
    case 2562: return launch_batched_t<NP, 256, 2>(p, sys, items, n_items, queue, shape.grid, smem, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

int launch_batched(const glisser_particles* pa, const BatchSystems& sys, const BatchItem* items,
                   const uint32_t* n_items, uint32_t* queue, uint32_t npl, uint32_t len,
                   const glisser_step_params* sp, const glisser_handoff* ho, const BatchShape& shape,
                   cudaStream_t stream)
{
    if (!pa || !sp || !ho || !items || !n_items || !queue) return GLISSER_E_INVALID;
    if (npl < 1 || npl > (uint32_t)MAX_PLANETS || !handoff_ok(ho)) return GLISSER_E_INVALID;
    if (((uintptr_t)sys.log & 15u) != 0 || (sys.log_stride * sizeof(double)) % 16 != 0) return GLISSER_E_INVALID;
    Common p;
    if (!fill_common(p, pa, sp, ho, npl, len)) return GLISSER_E_INVALID;
    size_t smem = timeblock_smem_bytes(npl, (int)p.chunk);
    cudaError_t e = npl == 5 ? launch_batched_np<4>(p, sys, items, n_items, queue, shape, smem, stream)
                             : launch_batched_np<0>(p, sys, items, n_items, queue, shape, smem, stream);
    if (e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof msg, "batched launch: %s", cudaGetErrorString(e));
        set_timeblock_error(msg);
        return GLISSER_E_CUDA;
    }
    return GLISSER_OK;
}

}  // namespace glisser
