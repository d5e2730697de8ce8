// Internal interface of the particle time-block kernels (shared by the
// C-ABI layer, the executor and the ensemble runner).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/glisser.h"

namespace glisser {

// Steps per planet-log chunk staged in shared memory (even, so that every
// chunk is a multiple of 16 bytes for the bulk copy).  Two chunk buffers per
// CTA: 32 steps keep the single-system kernel's 16 CTAs of 64 within shared
// memory with four planets (10.9 KB per CTA).
#ifndef GLISSER_LOG_CHUNK
#define GLISSER_LOG_CHUNK 32
#endif
constexpr int LOG_CHUNK = GLISSER_LOG_CHUNK;
// The ensemble kernel restages each system's log per tile and takes longer
// chunks (fewer waits per tile); 64 steps fit its 8 CTAs of 128 per SM
// (18.6 KB each with four planets).
#ifndef GLISSER_BATCH_LOG_CHUNK
#define GLISSER_BATCH_LOG_CHUNK 64
#endif
constexpr int BATCH_LOG_CHUNK = GLISSER_BATCH_LOG_CHUNK;
constexpr int MAX_PLANETS = 64;           // planets including the Sun
// Threads per CTA of the single-system kernel (a build-time tuning knob; the
// CTAs per SM its registers are sized for is GLISSER_TB_MIN_BLOCKS).
#ifndef GLISSER_TB_THREADS
#define GLISSER_TB_THREADS 64
#endif
constexpr int BLOCK_THREADS = GLISSER_TB_THREADS;

size_t timeblock_smem_bytes(uint32_t npl, int chunk = LOG_CHUNK);
uint32_t log_chunk_steps(uint32_t npl, uint32_t max_steps = LOG_CHUNK);

// Launches one time block; validates arguments and returns a GLISSER_* code.
const char* timeblock_error();
int launch_timeblock(const glisser_particles* pa, size_t n_alive, const glisser_planet_block* pl,
                     const glisser_step_params* sp, const glisser_handoff* ho, cudaStream_t stream);

// Ensembles: per-system planet blocks laid out at a fixed stride, and the
// (system, tile) work items of one block.
struct BatchSystems {
    const double* log;      // system s: log + s * log_stride (records of npl 3-vectors)
    size_t log_stride;      // doubles per system (multiple of 2: 16-byte aligned blocks)
    const double* m;        // [systems][npl]
    const double* rh;       // [systems][npl]
    const uint32_t* id;     // [systems][npl]
};

struct BatchItem {
    uint32_t system;
    uint32_t first;         // global particle index of the tile's first particle
    uint32_t count;         // particles in the tile (<= cta * ppt)
    uint32_t reserved;
};

struct BatchShape {
    int cta;                // threads per CTA: 64, 128 or 256
    int ppt;                // particles per thread: 1 or 2
    uint32_t grid;          // persistent CTAs (0: one wave at full occupancy)
};

int launch_batched(const glisser_particles* pa, const BatchSystems& sys, const BatchItem* items,
                   const uint32_t* n_items, uint32_t* queue, uint32_t npl, uint32_t len,
                   const glisser_step_params* sp, const glisser_handoff* ho, const BatchShape& shape,
                   cudaStream_t stream);

}  // namespace glisser
