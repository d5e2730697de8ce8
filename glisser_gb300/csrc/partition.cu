// Stable three-way partition of the particle arrays: unflagged particles
// first, then particles in encounter ((flags & 0xFE) == 0, flags != 0), then
// the rest.  Replaces the unstable thrust::partition calls of the reference
// executor (src/executor.cu:663-665, 784-790, 865-869) with a deterministic
// order, so the host mirror and every output file are reproducible.
//
// Three launches over tiles of TILE particles: per-tile category counts by
// warp ballot, one exclusive scan of the tile counts, and a scatter in which
// each tile recomputes its ranks and writes the 12 particle arrays to the
// output buffer.  HBM traffic is one read of the flags plus one read and one
// write of the 96-byte particle record.
#include <cuda.h>

#include <cstdio>
#include <mutex>

#include "timeblock.cuh"

namespace glisser {

namespace {

constexpr int TILE = 256;
constexpr int SCAN_THREADS = 1024;

__device__ __forceinline__ int category(uint16_t f)
{
    if (f == 0) return 0;
    if ((f & 0xFE) == 0) return 1;
    return 2;
}

// Per-tile counts of categories 0 and 1 into counts[2*tile + {0,1}].
__global__ void __launch_bounds__(TILE) count_kernel(const uint16_t* __restrict__ flags, uint32_t n, uint32_t* counts)
{
    __shared__ uint32_t warp_c[2][TILE / 32];
    uint32_t i = blockIdx.x * TILE + threadIdx.x;
    int cat = i < n ? category(flags[i]) : 2;
    unsigned b0 = __ballot_sync(0xffffffffu, cat == 0);
    unsigned b1 = __ballot_sync(0xffffffffu, cat == 1);
    if ((threadIdx.x & 31) == 0) {
        warp_c[0][threadIdx.x >> 5] = __popc(b0);
        warp_c[1][threadIdx.x >> 5] = __popc(b1);
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        uint32_t s = 0;
        for (int w = 0; w < TILE / 32; w++) s += warp_c[threadIdx.x][w];
        counts[2 * blockIdx.x + threadIdx.x] = s;
    }
}

// Exclusive scan of the per-tile counts in place (single CTA), totals out.
__global__ void __launch_bounds__(SCAN_THREADS) scan_kernel(uint32_t* counts, uint32_t ntiles, uint32_t* n0, uint32_t* n1)
{
    __shared__ uint32_t part[2][SCAN_THREADS];
    uint32_t per = (ntiles + SCAN_THREADS - 1) / SCAN_THREADS;
    uint32_t lo = threadIdx.x * per;
    uint32_t hi = min(lo + per, ntiles);
    uint32_t s0 = 0, s1 = 0;
    for (uint32_t t = lo; t < hi; t++) {
        s0 += counts[2 * t];
        s1 += counts[2 * t + 1];
    }
    part[0][threadIdx.x] = s0;
    part[1][threadIdx.x] = s1;
    __syncthreads();
    // Hillis-Steele inclusive scan over the 1024 partial sums
    for (int off = 1; off < SCAN_THREADS; off <<= 1) {
        uint32_t a0 = threadIdx.x >= (unsigned)off ? part[0][threadIdx.x - off] : 0;
        uint32_t a1 = threadIdx.x >= (unsigned)off ? part[1][threadIdx.x - off] : 0;
        __syncthreads();
        part[0][threadIdx.x] += a0;
        part[1][threadIdx.x] += a1;
        __syncthreads();
    }
    uint32_t b0 = part[0][threadIdx.x] - s0;
    uint32_t b1 = part[1][threadIdx.x] - s1;
    for (uint32_t t = lo; t < hi; t++) {
        uint32_t c0 = counts[2 * t], c1 = counts[2 * t + 1];
        counts[2 * t] = b0;
        counts[2 * t + 1] = b1;
        b0 += c0;
        b1 += c1;
    }
    if (threadIdx.x == SCAN_THREADS - 1) {
        *n0 = part[0][SCAN_THREADS - 1];
        *n1 = part[1][SCAN_THREADS - 1];
    }
}

__global__ void __launch_bounds__(TILE) scatter_kernel(glisser_particles in, glisser_particles out, uint32_t n,
                                                       const uint32_t* offsets, const uint32_t* n0p,
                                                       const uint32_t* n1p)
{
    __shared__ uint32_t warp_c[2][TILE / 32];
    uint32_t i = blockIdx.x * TILE + threadIdx.x;
    int cat = i < n ? category(in.flags[i]) : 3;
    unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned b0 = __ballot_sync(0xffffffffu, cat == 0);
    unsigned b1 = __ballot_sync(0xffffffffu, cat == 1);
    if (lane == 0) {
        warp_c[0][warp] = __popc(b0);
        warp_c[1][warp] = __popc(b1);
    }
    __syncthreads();
    if (i >= n) return;
    uint32_t before0 = 0, before1 = 0;
    for (unsigned w = 0; w < warp; w++) {
        before0 += warp_c[0][w];
        before1 += warp_c[1][w];
    }
    unsigned lt = (1u << lane) - 1u;
    uint32_t r0 = offsets[2 * blockIdx.x] + before0 + __popc(b0 & lt);
    uint32_t r1 = offsets[2 * blockIdx.x + 1] + before1 + __popc(b1 & lt);
    uint32_t n0 = *n0p, n1 = *n1p;
    uint32_t dst;
    if (cat == 0) dst = r0;
    else if (cat == 1) dst = n0 + r1;
    else dst = n0 + n1 + (i - r0 - r1);
    out.rx[dst] = in.rx[i]; out.ry[dst] = in.ry[i]; out.rz[dst] = in.rz[i];
    out.vx[dst] = in.vx[i]; out.vy[dst] = in.vy[i]; out.vz[dst] = in.vz[i];
    out.ax[dst] = in.ax[i]; out.ay[dst] = in.ay[i]; out.az[dst] = in.az[i];
    out.flags[dst] = in.flags[i];
    out.deathtime_index[dst] = in.deathtime_index[i];
    out.id[dst] = in.id[i];
}

__global__ void copy_range_kernel(glisser_particles src, glisser_particles dst, uint32_t begin, uint32_t end)
{
    uint32_t i = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    dst.rx[i] = src.rx[i]; dst.ry[i] = src.ry[i]; dst.rz[i] = src.rz[i];
    dst.vx[i] = src.vx[i]; dst.vy[i] = src.vy[i]; dst.vz[i] = src.vz[i];
    dst.ax[i] = src.ax[i]; dst.ay[i] = src.ay[i]; dst.az[i] = src.az[i];
    dst.flags[i] = src.flags[i];
    dst.deathtime_index[i] = src.deathtime_index[i];
    dst.id[i] = src.id[i];
}

}  // namespace

// Copies particles [begin, end) between two particle buffers.
int launch_copy_range(const glisser_particles* src, const glisser_particles* dst, size_t begin, size_t end,
                      cudaStream_t stream)
{
    if (end <= begin) return GLISSER_OK;
    uint32_t n = (uint32_t)(end - begin);
    copy_range_kernel<<<(n + 255) / 256, 256, 0, stream>>>(*src, *dst, (uint32_t)begin, (uint32_t)end);
    return cudaGetLastError() == cudaSuccess ? GLISSER_OK : GLISSER_E_CUDA;
}

size_t partition_scratch_bytes(size_t n)
{
    size_t tiles = (n + TILE - 1) / TILE;
    return 2 * tiles * sizeof(uint32_t) + 64;
}

int launch_partition(const glisser_particles* in, const glisser_particles* out, size_t n, void* scratch,
                     uint32_t* n0, uint32_t* n1, cudaStream_t stream)
{
    if (!in || !out || !scratch || !n0 || !n1) return GLISSER_E_INVALID;
    if (n > 0xFFFFFF00ull) return GLISSER_E_INVALID;
    if (n == 0) {
        cudaMemsetAsync(n0, 0, sizeof(uint32_t), stream);
        cudaMemsetAsync(n1, 0, sizeof(uint32_t), stream);
        return cudaGetLastError() == cudaSuccess ? GLISSER_OK : GLISSER_E_CUDA;
    }
    uint32_t tiles = (uint32_t)((n + TILE - 1) / TILE);
    uint32_t* counts = reinterpret_cast<uint32_t*>(scratch);
    count_kernel<<<tiles, TILE, 0, stream>>>(in->flags, (uint32_t)n, counts);
    scan_kernel<<<1, SCAN_THREADS, 0, stream>>>(counts, tiles, n0, n1);
    scatter_kernel<<<tiles, TILE, 0, stream>>>(*in, *out, (uint32_t)n, counts, n0, n1);
    return cudaGetLastError() == cudaSuccess ? GLISSER_OK : GLISSER_E_CUDA;
}


// ---------------------------------------------------------------------------
// Partition without allocation.
//
// For callers that must not allocate device memory at all: a host program
// that runs inside another framework's memory pool or under a fixed device
// budget, where a cudaMalloc would either be refused or would synchronise the
// whole device and stall work the caller has in flight.  Such a caller still
// owns the particle buffers and the two count words; the per-tile counts
// that glisser_partition keeps in caller-provided scratch live here in a
// file-scope device array instead.
//
// NOALLOC_MAX_PARTICLES bounds n: 2 counts per 256-particle tile, 256 KiB in
// all, resident on every GPU that loads the library until the process exits.
// Every call shares that array and leaves the last call's counts in it.  No
// entry needs clearing before a call (count_kernel writes every tile's counts
// before scan_kernel reads them), but two calls whose work overlaps on the
// GPU, on one stream or several, race on the array and corrupt each other.
constexpr size_t NOALLOC_MAX_PARTICLES = 8u << 20;
constexpr size_t NOALLOC_TILES = NOALLOC_MAX_PARTICLES / TILE;

static __device__ __align__(256) uint32_t g_noalloc_counts[2 * NOALLOC_TILES];

namespace {

// Device address of g_noalloc_counts per device.  In host code the array's
// name is only a host-side stand-in; the address kernels need comes from
// cudaGetSymbolAddress, resolved with that device current.  The address
// belongs to the context the library's module was loaded into, so it is
// cached together with that context (the driver's cuCtxGetCurrent, reached
// through the runtime's entry-point query so that the library needs no link
// to the driver library) and looked up again when the current context
// differs: after a cudaDeviceReset, or under another context of the same
// device, a call resolves the array afresh instead of using a stale address.
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
uint32_t* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};
CUcontext g_noalloc_ctx[NOALLOC_MAX_DEVICES] = {};

using CtxGetCurrent = CUresult (*)(CUcontext*);

CtxGetCurrent ctx_get_current()
{
    static CtxGetCurrent fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<CtxGetCurrent>(f);
    }();
    return fn;
}

CUcontext current_context()
{
    CUcontext c = nullptr;
    CtxGetCurrent fn = ctx_get_current();
    if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
    return c;
}

int noalloc_scratch(uint32_t** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) return GLISSER_E_CUDA;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    const CUcontext ctx = current_context();
    if (!g_noalloc_ptr[dev] || !ctx || ctx != g_noalloc_ctx[dev]) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_noalloc_counts) != cudaSuccess || !ptr) return GLISSER_E_CUDA;
        g_noalloc_ptr[dev] = static_cast<uint32_t*>(ptr);
        g_noalloc_ctx[dev] = current_context();   // the context the lookup ran in
    }
    *out = g_noalloc_ptr[dev];
    return GLISSER_OK;
}

}  // namespace

size_t partition_noalloc_max_particles() { return NOALLOC_MAX_PARTICLES; }

int launch_partition_noalloc(const glisser_particles* in, const glisser_particles* out, size_t n, uint32_t* n0,
                             uint32_t* n1, cudaStream_t stream)
{
    if (!in || !out || !n0 || !n1) return GLISSER_E_INVALID;
    if (n > NOALLOC_MAX_PARTICLES) return GLISSER_E_INVALID;
    uint32_t* counts = nullptr;
    int rc = noalloc_scratch(&counts);
    if (rc != GLISSER_OK) return rc;
    if (n == 0) {
        cudaMemsetAsync(n0, 0, sizeof(uint32_t), stream);
        cudaMemsetAsync(n1, 0, sizeof(uint32_t), stream);
        return cudaGetLastError() == cudaSuccess ? GLISSER_OK : GLISSER_E_CUDA;
    }
    uint32_t tiles = (uint32_t)((n + TILE - 1) / TILE);
    count_kernel<<<tiles, TILE, 0, stream>>>(in->flags, (uint32_t)n, counts);
    scan_kernel<<<1, SCAN_THREADS, 0, stream>>>(counts, tiles, n0, n1);
    scatter_kernel<<<tiles, TILE, 0, stream>>>(*in, *out, (uint32_t)n, counts, n0, n1);
    return cudaGetLastError() == cudaSuccess ? GLISSER_OK : GLISSER_E_CUDA;
}

}  // namespace glisser
