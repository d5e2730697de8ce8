// Particle time-block kernels: the GB300 replacement of MVSKernel
// (src/wh.cu:15-207) and its launch (src/wh.cu:344-395).
//
// One thread keeps the state of its particle(s) -- r, v and the flag word --
// in registers for the whole block of `len` steps (the acceleration and the
// deathtime index are stored at the particle's last step); the arrays are
// structure-of-arrays FP64 so every load and store is a fully coalesced
// 8-byte-per-lane access.  The planet log (per step: h0, then the planet
// positions) is staged into shared memory in chunks of `chunk` steps by bulk
// TMA copies (cp.async.bulk ... mbarrier::complete_tx), double buffered, and
// read from there as warp-wide broadcasts.  The drift is the universal-
// variable solver of kepler.cuh.  Flag semantics follow the reference kernel
// (src/wh.cu:132-176): the first planet inside its radius marks the particle
// with (planet id << 8) | 0x01, the Sun's radius overrides with 0x01 and the
// outer limit with 0x02, and a flagged particle stops for the rest of the
// block with deathtime_index = last integrated step + 1.  The block epilogue
// optionally applies KillEncounterKernel (src/executor.cu:63-78) and appends
// every particle whose flags changed to the hand-off list, compacted with a
// warp ballot and one atomic per warp.
//
// Two launches share the tile routine:
//  * timeblock_kernel: one system, one tile of BLOCK_THREADS particles per CTA;
//  * batched_kernel: many systems (ensembles), persistent CTAs that pop
//    (system, tile) items from a device work queue and stage each item's own
//    planet log; CTA size and particles per thread are template parameters
//    chosen by the autotuner.
#include <cstdio>

#include "timeblock_kernel.cuh"

namespace glisser {

using namespace tile;

namespace {

thread_local char g_err[256];

}  // namespace

uint32_t log_chunk_steps(uint32_t npl, uint32_t max_steps)
{
    // as many steps as fit two buffers in 200 KB, at most max_steps, even
    size_t rec_bytes = 3ull * npl * sizeof(double);
    size_t fit = (200u * 1024u) / (2 * rec_bytes);
    return (uint32_t)(fit < (size_t)max_steps ? fit : (size_t)max_steps) & ~1u;
}

size_t timeblock_smem_bytes(uint32_t npl, int chunk) { return 2ull * (size_t)chunk * 3u * npl * sizeof(double); }

const char* timeblock_error() { return g_err; }


int launch_timeblock(const glisser_particles* pa, size_t n_alive, const glisser_planet_block* pl,
                     const glisser_step_params* sp, const glisser_handoff* ho, cudaStream_t stream)
{
    if (!pa || !pl || !sp || !ho) return GLISSER_E_INVALID;
    if (pl->npl < 1 || pl->npl > (uint32_t)MAX_PLANETS) return GLISSER_E_INVALID;
    if (n_alive > 0xFFFFFFF0ull) return GLISSER_E_INVALID;
    if (!handoff_ok(ho)) return GLISSER_E_INVALID;
    if (!(sp->dt > 0) || !(sp->outer_radius >= 0)) return GLISSER_E_INVALID;
    if (!(sp->kepler_tol == 0 || (sp->kepler_tol >= 1e-16 && sp->kepler_tol <= 1e-8))) return GLISSER_E_INVALID;
    if (sp->kill_encounters < GLISSER_ENCOUNTERS_KEEP || sp->kill_encounters > GLISSER_ENCOUNTERS_ROLLBACK)
        return GLISSER_E_INVALID;
    if (sp->kick != GLISSER_KICK_FLOAT_FLOAT && sp->kick != GLISSER_KICK_FP64) return GLISSER_E_INVALID;
    if (pl->len > 0) {
        if (!pl->log || !pl->m || !pl->id || !pl->rh) return GLISSER_E_INVALID;
        if (((uintptr_t)pl->log & 15u) != 0) return GLISSER_E_INVALID;
        if (pl->capacity < ((pl->len + 1u) & ~1u)) return GLISSER_E_INVALID;
    }
    if (n_alive == 0) return GLISSER_OK;

    Common p;
    if (!fill_common(p, pa, sp, ho, pl->npl, pl->len)) return GLISSER_E_INVALID;
    size_t smem = timeblock_smem_bytes(pl->npl, (int)p.chunk);
    uint32_t n = (uint32_t)n_alive;
    cudaError_t e;
    if (sp->starter == GLISSER_STARTER_LEARNED && p.mlp)
        e = launch_timeblock_learned(p, pl, n, smem, stream);
    else if (p.kick64)
        e = launch_timeblock_kick64(p, pl, n, smem, stream);
    else
        e = launch_variant<false, false>(p, pl, n, smem, stream);
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof g_err, "time-block launch: %s", cudaGetErrorString(e));
        return GLISSER_E_CUDA;
    }
    return GLISSER_OK;
}

void set_timeblock_error(const char* msg) { snprintf(g_err, sizeof g_err, "%s", msg); }

}  // namespace glisser
