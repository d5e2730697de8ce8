// Internal interface of the particle time-block kernels (shared by the
// C-ABI layer and the executor).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/glisser.h"

namespace glisser {

// Steps per planet-log chunk staged in shared memory (even, so that every
// chunk is a multiple of 16 bytes for the bulk copy).
constexpr int LOG_CHUNK = 128;
constexpr int MAX_PLANETS = 64;           // planets including the Sun
constexpr int BLOCK_THREADS = 128;

size_t timeblock_smem_bytes(uint32_t npl, int chunk = LOG_CHUNK);

// Launches one time block; validates arguments and returns a GLISSER_* code.
const char* timeblock_error();
int launch_timeblock(const glisser_particles* pa, size_t n_alive, const glisser_planet_block* pl,
                     const glisser_step_params* sp, const glisser_handoff* ho, cudaStream_t stream);

}  // namespace glisser
