// Device track-snapshot records (host interface of track.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/glisser.h"

namespace glisser {

// Centre the elements are taken about: G*mass and position / velocity.
struct TrackFrame {
    double cm;
    double cr[3], cv[3];
};

// uint32 words of scratch launch_track_records needs for ids up to max_id.
size_t track_scratch_words(uint32_t max_id);

// Writes the 28-byte records (id, a, e, i, capom, om, f as float32) of
// particles [0, n) into `out` (n * 28 bytes, device) ordered by id, on
// `stream`.  The ids must be distinct and at most max_id.
cudaError_t launch_track_records(const glisser_particles* pa, uint32_t n, uint32_t max_id, const TrackFrame& fr,
                                 uint32_t* scratch, void* out, cudaStream_t stream);

}  // namespace glisser
