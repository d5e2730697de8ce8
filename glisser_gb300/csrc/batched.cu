// Ensemble time-block kernel: many independent systems (each its own
// planets and particle range) in one persistent launch.  CTAs pop
// (system, tile) items from a device work queue (one atomic per item), load
// that system's planet constants, and run the same tile routine as the
// single-system kernel, staging the item's own planet log through the bulk-
// TMA double buffer.  Items of one system are consecutive, so neighbouring
// CTAs share that system's log in L2.  The CTA size (64/128/256) and the
// particles per thread (1/2) are template parameters picked by the autotuner.
#include <cstdio>

#include "batched_kernel.cuh"

namespace glisser {

using namespace tile;

const char* timeblock_error();
void set_timeblock_error(const char* msg);

int launch_batched(const glisser_particles* pa, const BatchSystems& sys, const BatchItem* items,
                   const uint32_t* n_items, uint32_t* queue, uint32_t npl, uint32_t len,
                   const glisser_step_params* sp, const glisser_handoff* ho, const BatchShape& shape,
                   cudaStream_t stream)
{
    if (!pa || !sp || !ho || !items || !n_items || !queue) return GLISSER_E_INVALID;
    if (npl < 1 || npl > (uint32_t)MAX_PLANETS || !handoff_ok(ho)) return GLISSER_E_INVALID;
    if (!(sp->kepler_tol == 0 || (sp->kepler_tol >= 1e-16 && sp->kepler_tol <= 1e-8))) return GLISSER_E_INVALID;
    if (sp->kill_encounters < GLISSER_ENCOUNTERS_KEEP || sp->kill_encounters > GLISSER_ENCOUNTERS_ROLLBACK)
        return GLISSER_E_INVALID;
    if (sp->kick != GLISSER_KICK_FLOAT_FLOAT && sp->kick != GLISSER_KICK_FP64) return GLISSER_E_INVALID;
    if (((uintptr_t)sys.log & 15u) != 0 || (sys.log_stride * sizeof(double)) % 16 != 0) return GLISSER_E_INVALID;
    Common p;
    if (!fill_common(p, pa, sp, ho, npl, len, BATCH_LOG_CHUNK)) return GLISSER_E_INVALID;
    size_t smem = timeblock_smem_bytes(npl, (int)p.chunk);
    cudaError_t e;
    const bool learned = sp->starter == GLISSER_STARTER_LEARNED && p.mlp;
    if (learned && p.kick64)
        e = launch_batched_learned_kick64(p, sys, items, n_items, queue, npl, shape, smem, stream);
    else if (learned)
        e = launch_batched_learned(p, sys, items, n_items, queue, npl, shape, smem, stream);
    else if (p.kick64)
        e = launch_batched_kick64(p, sys, items, n_items, queue, npl, shape, smem, stream);
    else
        e = launch_batched_variant<false, false>(p, sys, items, n_items, queue, npl, shape, smem, stream);
    if (e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof msg, "batched launch: %s", cudaGetErrorString(e));
        set_timeblock_error(msg);
        return GLISSER_E_CUDA;
    }
    return GLISSER_OK;
}

}  // namespace glisser
