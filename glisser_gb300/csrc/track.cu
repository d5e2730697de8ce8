// Track snapshots on the device: the particle part of save_binary_track
// (src/data.cpp:718-815) -- alive particles ordered by id, each converted to
// orbital elements in FP64 (to_elements, src/convert.cpp:310-463) and packed
// as a 28-byte record (u32 id, six float32) -- written into a staging buffer
// in its final file order, ready for one device-to-host copy.
//
// Ordering by id without a sort: the ids present mark a bitmap (one bit per
// id up to the largest id), a scan of the bitmap's word popcounts gives each
// word's rank base, and a particle's slot is that base plus the popcount of
// the lower bits of its word.  Work and memory are O(max id / 32) on top of
// O(n), so the executor uses this path when the ids are dense (the state
// files number particles 0..n-1) and keeps the host writer otherwise.
//
// The element formulas and their operation order are the host
// restatement's (orbits.cpp to_elements); this translation unit is compiled
// without FMA contraction, so records differ from the host writer's only
// through the device transcendentals (acos, asin, atan2, sincos), and after
// rounding to float32 almost always not at all.
#include "track.h"

namespace glisser {
namespace {

constexpr int SCAN_BLOCK = 1024;

__global__ void mark_kernel(const uint32_t* __restrict__ id, uint32_t n, uint32_t max_id, uint32_t* __restrict__ bitmap)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t v = id[i];
    if (v > max_id) return;        // outside the bitmap: the caller guarantees it never happens
    atomicOr(&bitmap[v >> 5], 1u << (v & 31u));
}

// Per SCAN_BLOCK words: exclusive prefix of the popcounts within the block
// (pre) and the block's total (blk).
__global__ void __launch_bounds__(SCAN_BLOCK) word_scan_kernel(const uint32_t* __restrict__ bitmap, uint32_t words,
                                                               uint32_t* __restrict__ pre, uint32_t* __restrict__ blk)
{
    __shared__ uint32_t warp_sum[SCAN_BLOCK / 32];
    const uint32_t w = blockIdx.x * SCAN_BLOCK + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t c = w < words ? __popc(bitmap[w]) : 0u;
    uint32_t x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = warp_sum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= (uint32_t)o) s += y;
        }
        warp_sum[lane] = s;       // inclusive over warps
    }
    __syncthreads();
    const uint32_t base = warp ? warp_sum[warp - 1] : 0u;
    if (w < words) pre[w] = base + x - c;
    if (threadIdx.x == SCAN_BLOCK - 1) blk[blockIdx.x] = base + x;
}

// Exclusive scan of the block totals in place (one CTA, sequential over
// chunks of SCAN_BLOCK with a carry).
__global__ void __launch_bounds__(SCAN_BLOCK) block_scan_kernel(uint32_t* __restrict__ blk, uint32_t nblk)
{
    __shared__ uint32_t warp_sum[SCAN_BLOCK / 32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (uint32_t off = 0; off < nblk; off += SCAN_BLOCK) {
        const uint32_t k = off + threadIdx.x;
        const uint32_t c = k < nblk ? blk[k] : 0u;
        uint32_t x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) warp_sum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t s = warp_sum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= (uint32_t)o) s += y;
            }
            warp_sum[lane] = s;
        }
        __syncthreads();
        const uint32_t base = carry + (warp ? warp_sum[warp - 1] : 0u);
        if (k < nblk) blk[k] = base + x - c;
        __syncthreads();
        if (threadIdx.x == SCAN_BLOCK - 1) carry = base + x;
        __syncthreads();
    }
}

struct El {
    double a, e, i, capom, om, f;
};

// to_elements (orbits.cpp, restating src/convert.cpp:310-463).
__device__ El to_elements_dev(double mu, double x, double y, double z, double vx, double vy, double vz)
{
    El el;
    const double pi = 2.0 * asin(1.0);
    const double prec = 1.0e-13;
    const double hx = y * vz - z * vy, hy = z * vx - x * vz, hz = x * vy - y * vx;
    const double hsq = hx * hx + hy * hy + hz * hz;
    if (!(hsq > prec)) {
        const double d = sqrt(x * x + y * y + z * z);
        el.a = d;
        el.e = HUGE_VAL;
        el.i = asin(z / d);
        el.capom = atan2(y, x);
        el.om = HUGE_VAL;
        el.f = HUGE_VAL;
        return el;
    }
    el.i = acos(hz / sqrt(hsq));
    if (fabs(el.i) < prec || fabs(pi - fabs(el.i)) < prec) el.capom = 0.0;
    else el.capom = atan2(hx, -hy);
    const double vsq = vx * vx + vy * vy + vz * vz;
    const double vdotr = x * vx + y * vy + z * vz;
    const double rr = sqrt(x * x + y * y + z * z);
    const double xh = x / rr, yh = y / rr, zh = z / rr;
    double ny, nx;
    sincos(el.capom, &ny, &nx);
    const double fac = vsq * rr - mu;
    const double px = fac * xh - vdotr * vx, py = fac * yh - vdotr * vy, pz = fac * zh - vdotr * vz;
    el.e = sqrt(px * px + py * py + pz * pz) / mu;
    const bool planar = el.i < prec || pi - el.i < prec;
    if (fabs(el.e) < prec) {
        el.om = 0.0;
    } else if (planar) {
        el.om = atan2(py, px);
    } else {
        el.om = acos(((nx * px + ny * py) / mu) / el.e);
        if (fabs(pz) > prec) el.om *= fabs(pz) / pz;
    }
    const double energy = vsq / 2.0 - mu / rr;
    const double sgn = vdotr / fabs(vdotr);
    if (fabs(energy) < prec) {
        el.a = 0.5 * hsq / mu;
        el.f = fabs(vdotr) < prec ? 0.0 : 2.0 * acos(sqrt(el.a / rr)) * sgn;
    } else if (energy > 0.0) {
        el.a = -0.5 * mu / energy;
        el.f = fabs(vdotr) < prec ? 0.0 : acos((el.a * (1.0 - el.e * el.e) / rr - 1.0) / el.e) * sgn;
    } else {
        el.a = -0.5 * mu / energy;
        if (fabs(el.e) > prec) {
            if (fabs(vdotr) < prec) {
                el.f = rr < el.a ? 0.0 : pi;
            } else {
                el.f = acos((el.a * (1.0 - el.e * el.e) / rr - 1.0) / el.e) * sgn;
                if (isnan(el.f)) el.f = rr < el.a ? 0.0 : pi;
            }
        } else {
            el.f = acos((x * nx + y * ny) / rr);
            if (fabs(z) > prec) el.f *= fabs(z) / z;
            else if (planar) el.f = atan2(y, x) * cos(el.i);
        }
    }
    return el;
}

__global__ void record_kernel(glisser_particles pa, uint32_t n, uint32_t max_id, TrackFrame fr,
                              const uint32_t* __restrict__ bitmap, const uint32_t* __restrict__ pre,
                              const uint32_t* __restrict__ blk, uint32_t* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = pa.id[i];
    if (id > max_id) return;
    const uint32_t w = id >> 5;
    const uint32_t slot = blk[w / SCAN_BLOCK] + pre[w] + __popc(bitmap[w] & ((1u << (id & 31u)) - 1u));
    const El el = to_elements_dev(fr.cm, pa.rx[i] - fr.cr[0], pa.ry[i] - fr.cr[1], pa.rz[i] - fr.cr[2],
                                  pa.vx[i] - fr.cv[0], pa.vy[i] - fr.cv[1], pa.vz[i] - fr.cv[2]);
    uint32_t* rec = out + 7 * (size_t)slot;
    rec[0] = id;
    rec[1] = __float_as_uint((float)el.a);
    rec[2] = __float_as_uint((float)el.e);
    rec[3] = __float_as_uint((float)el.i);
    rec[4] = __float_as_uint((float)el.capom);
    rec[5] = __float_as_uint((float)el.om);
    rec[6] = __float_as_uint((float)el.f);
}

}  // namespace

size_t track_scratch_words(uint32_t max_id)
{
    const size_t words = ((size_t)max_id >> 5) + 1;
    const size_t nblk = (words + SCAN_BLOCK - 1) / SCAN_BLOCK;
    return 2 * words + nblk;
}

cudaError_t launch_track_records(const glisser_particles* pa, uint32_t n, uint32_t max_id, const TrackFrame& fr,
                                 uint32_t* scratch, void* out, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    const uint32_t words = (max_id >> 5) + 1;
    const uint32_t nblk = (words + SCAN_BLOCK - 1) / SCAN_BLOCK;
    uint32_t* bitmap = scratch;
    uint32_t* pre = scratch + words;
    uint32_t* blk = pre + words;
    cudaError_t e = cudaMemsetAsync(bitmap, 0, (size_t)words * sizeof(uint32_t), stream);
    if (e != cudaSuccess) return e;
    mark_kernel<<<(n + 255) / 256, 256, 0, stream>>>(pa->id, n, max_id, bitmap);
    word_scan_kernel<<<nblk, SCAN_BLOCK, 0, stream>>>(bitmap, words, pre, blk);
    block_scan_kernel<<<1, SCAN_BLOCK, 0, stream>>>(blk, nblk);
    record_kernel<<<(n + 127) / 128, 128, 0, stream>>>(*pa, n, max_id, fr, bitmap, pre, blk,
                                                       static_cast<uint32_t*>(out));
    return cudaGetLastError();
}

}  // namespace glisser
