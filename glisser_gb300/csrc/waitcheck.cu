// Self-test of the bounded mbarrier wait the time-block kernels stage their
// planet logs with: one CTA arms a barrier for 16 bytes of transaction that
// are never issued (nothing will complete the phase) and waits with the same
// routine and a caller-chosen limit.  The wait must give up, report the
// staging-timeout status bit and let the kernel end normally, leaving the
// context usable.  No copy is in flight at any time.
#include <cstdio>

#include "tile.cuh"

namespace glisser {
namespace {

using namespace tile;

__global__ void wait_check_kernel(uint64_t limit_ns, uint32_t* status, unsigned long long* elapsed_ns)
{
    __shared__ uint64_t bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    mbar_fence_init();
    mbar_expect_tx(&bar, 16);                 // arrival done, 16 bytes still expected
    const uint64_t t0 = global_ns();
    const bool ok = mbar_wait_bounded(&bar, 0, limit_ns);
    *elapsed_ns = global_ns() - t0;
    if (!ok) atomicOr(status, GLISSER_STATUS_LOG_TIMEOUT);
}

}  // namespace

int wait_check(double limit_seconds, uint32_t* status_out, double* elapsed_out)
{
    if (!(limit_seconds > 0) || limit_seconds > 10.0 || !status_out) return GLISSER_E_INVALID;
    uint32_t* d_status = nullptr;
    unsigned long long* d_el = nullptr;
    if (cudaMalloc(&d_status, sizeof(uint32_t)) != cudaSuccess) return GLISSER_E_NOMEM;
    if (cudaMalloc(&d_el, sizeof(unsigned long long)) != cudaSuccess) {
        cudaFree(d_status);
        return GLISSER_E_NOMEM;
    }
    int rc = GLISSER_OK;
    unsigned long long el = 0;
    if (cudaMemset(d_status, 0, sizeof(uint32_t)) != cudaSuccess) rc = GLISSER_E_CUDA;
    if (rc == GLISSER_OK) {
        wait_check_kernel<<<1, 32>>>((uint64_t)(limit_seconds * 1e9), d_status, d_el);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = GLISSER_E_CUDA;
    }
    if (rc == GLISSER_OK && (cudaMemcpy(status_out, d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
                             cudaMemcpy(&el, d_el, sizeof el, cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = GLISSER_E_CUDA;
    if (elapsed_out) *elapsed_out = (double)el * 1e-9;
    cudaFree(d_status);
    cudaFree(d_el);
    return rc;
}

}  // namespace glisser
