// Device residency of the learned-starter weights.
#include <cstring>
#include <stdexcept>
#include <vector>

#include <cuda_runtime.h>

#include "mlp.cuh"

namespace glisser {

// The weights blob is the byte image of MlpDev (written by the trainer).
void* mlp_upload(const std::vector<uint8_t>& blob)
{
    if (blob.size() != sizeof(MlpDev)) throw std::runtime_error("learned-starter weights blob has the wrong size");
    void* d = nullptr;
    if (cudaMalloc(&d, sizeof(MlpDev)) != cudaSuccess) throw std::runtime_error("cudaMalloc for the MLP weights failed");
    if (cudaMemcpy(d, blob.data(), sizeof(MlpDev), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        throw std::runtime_error("MLP weights upload failed");
    }
    return d;
}

void mlp_free(void* d)
{
    if (d) cudaFree(d);
}

size_t mlp_blob_bytes() { return sizeof(MlpDev); }

}  // namespace glisser
