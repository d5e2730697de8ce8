// Particle time-block kernel: the GB300 replacement of MVSKernel
// (src/wh.cu:15-207) and its launch (src/wh.cu:344-395).
//
// One thread per particle keeps r, v, a and the flag word in registers for
// the whole block of `len` steps; the particle arrays are structure-of-arrays
// FP64 so every load and store is a fully coalesced 8-byte-per-lane access.
// The planet log (per step: h0, then the planet positions) is staged into
// shared memory in chunks of `chunk` steps by bulk TMA copies
// (cp.async.bulk ... mbarrier::complete_tx), double buffered, and read
// from there as warp-wide broadcasts.  The drift is the universal-variable
// solver of kepler.cuh.  Flag semantics follow the reference kernel
// (src/wh.cu:132-176): the first planet inside its radius marks the particle
// with (planet id << 8) | 0x01, the Sun's radius overrides with 0x01 and the
// outer limit with 0x02, and a flagged particle stops for the rest of the
// block with deathtime_index = last integrated step + 1.  The block epilogue
// optionally applies KillEncounterKernel (src/executor.cu:63-78) and appends
// every particle whose flags changed to the hand-off list, compacted with a
// warp ballot and one atomic per warp.
#include <cstdio>

#include "kepler.cuh"
#include "timeblock.cuh"

namespace glisser {

namespace {

struct KParams {
    glisser_particles pa;
    uint32_t n;
    const double* log;
    const double* m;
    const uint32_t* pid;
    const double* rh;
    uint32_t npl;
    uint32_t len;
    uint32_t chunk;
    double dt;
    double outer2;
    int starter;
    int kill;
    const MlpDev* mlp;
    glisser_handoff ho;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Bounded wait: ~2^22 polls (each poll may itself suspend briefly).
constexpr uint32_t WAIT_POLLS = 1u << 22;

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity)
{
    for (uint32_t k = 0; k < WAIT_POLLS; k++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Issues the copy of log chunk c into buffer (c & 1).  Bytes are rounded up
// to an even number of steps; the caller guarantees capacity for it.
__device__ __forceinline__ void issue_chunk(const KParams& p, double* buf, uint64_t* bar, uint32_t c, uint32_t rec)
{
    uint32_t first = c * p.chunk;
    uint32_t steps = min(p.chunk, p.len - first);
    steps = (steps + 1u) & ~1u;
    uint32_t bytes = steps * rec * 8u;
    mbar_expect_tx(bar, bytes);
    bulk_copy_g2s(buf, p.log + (size_t)first * rec, bytes, bar);
}

// Acceleration from planet j and its encounter test (src/wh.cu:145-160):
// the first planet inside its radius wins (flags == 0 guard).
__device__ __forceinline__ void planet_kick(const double* L, int j, double rx, double ry, double rz, double& ax,
                                            double& ay, double& az, uint16_t& flags, const double* s_m,
                                            const double* s_rh2, const uint32_t* s_id)
{
    double dx = rx - L[3 * j];
    double dy = ry - L[3 * j + 1];
    double dz = rz - L[3 * j + 2];
    double rad = fma(dx, dx, fma(dy, dy, dz * dz));
    if (lt_nonneg(rad, s_rh2[j]) && flags == 0) flags = (uint16_t)((s_id[j] << 8) | 0x0001);
    double inv = rsqrt_fast46(rad);
    double fac = s_m[j] * (inv * inv * inv);
    ax = fma(-dx, fac, ax);
    ay = fma(-dy, fac, ay);
    az = fma(-dz, fac, az);
}

// CTAs per SM the register allocation is sized for (FP64-pipe bound: more
// resident warps only help cover FP64 latency)
#ifndef GLISSER_TB_MIN_BLOCKS
#define GLISSER_TB_MIN_BLOCKS 4
#endif

template <int NP>
__global__ void __launch_bounds__(BLOCK_THREADS, GLISSER_TB_MIN_BLOCKS) timeblock_kernel(const KParams p)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ double s_m[MAX_PLANETS];
    __shared__ double s_rh2[MAX_PLANETS];
    __shared__ uint32_t s_id[MAX_PLANETS];
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ volatile int s_abort;

    const int np = NP > 0 ? NP : (int)p.npl - 1;
    const uint32_t rec = 3u * (uint32_t)(np + 1);
    double* buf[2] = { reinterpret_cast<double*>(smem_raw), reinterpret_cast<double*>(smem_raw) + (size_t)p.chunk * rec };
    const uint32_t tid = threadIdx.x;
    const uint32_t nchunks = (p.len + p.chunk - 1) / p.chunk;

    if (tid < p.npl) {
        s_m[tid] = p.m[tid];
        s_rh2[tid] = p.rh[tid] * p.rh[tid];
        s_id[tid] = p.pid[tid];
    }
    if (tid == 0) {
        s_abort = 0;
        mbar_init(&s_bar[0], 1);
        mbar_init(&s_bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    int pend[2] = { -1, -1 };    // chunk in flight per buffer (thread 0 only)
    if (tid == 0) {
        for (uint32_t c = 0; c < nchunks && c < 2; c++) {
            issue_chunk(p, buf[c], &s_bar[c], c, rec);
            pend[c] = (int)c;
        }
    }

    const uint32_t i = blockIdx.x * BLOCK_THREADS + tid;
    const bool active = i < p.n;
    double rx = 0, ry = 0, rz = 0, vx = 0, vy = 0, vz = 0, ax = 0, ay = 0, az = 0;
    uint16_t flags = 0xFFFF;
    if (active) {
        rx = p.pa.rx[i]; ry = p.pa.ry[i]; rz = p.pa.rz[i];
        vx = p.pa.vx[i]; vy = p.pa.vy[i]; vz = p.pa.vz[i];
        ax = p.pa.ax[i]; ay = p.pa.ay[i]; az = p.pa.az[i];
        flags = p.pa.flags[i];
    }
    const uint16_t flags0 = flags;
    uint32_t dti = 0;
    uint32_t evals = 0;
    const double hdt = p.dt * 0.5;
    const double dt2mu = p.dt * p.dt * s_m[0];
    const double mu = s_m[0];
    const double rh2_sun = s_rh2[0];
    // Kick-drift-kick with the two half kicks between consecutive steps
    // merged into one full kick (v += a dt); a particle takes the closing half
    // kick when it is flagged or the block ends, so its stored velocity is
    // always at a step boundary.  |r|^2 from the Sun/outer test is the next
    // drift's r0^2.
    if (flags == 0 && p.len > 0) {
        vx = fma(ax, hdt, vx);
        vy = fma(ay, hdt, vy);
        vz = fma(az, hdt, vz);
    }
    double r2 = fma(rx, rx, fma(ry, ry, rz * rz));

    for (uint32_t c = 0; c < nchunks; c++) {
        const uint32_t b = c & 1u;
        if (!s_abort) {
            if (!mbar_wait_bounded(&s_bar[b], (c >> 1) & 1u)) {
                s_abort = 1;
                atomicOr(p.ho.status, GLISSER_STATUS_LOG_TIMEOUT);
            }
        }
        __syncthreads();
        if (s_abort) break;
        pend[b] = -1;
        const double* L0 = buf[b];
        const uint32_t first = c * p.chunk;
        const uint32_t steps = min(p.chunk, p.len - first);
        for (uint32_t s = 0; s < steps; s++) {
            if (flags != 0) continue;
            DriftResult d = kepler_drift(rx, ry, rz, vx, vy, vz, r2, p.dt, mu, dt2mu, p.starter, p.mlp);
            flags = d.flags;
            evals += d.evals;
            const double* L = L0 + (size_t)s * rec;
            ax = L[0]; ay = L[1]; az = L[2];
            if constexpr (NP > 0) {
#pragma unroll
                for (int j = 1; j <= NP; j++)
                    planet_kick(L, j, rx, ry, rz, ax, ay, az, flags, s_m, s_rh2, s_id);
            } else {
                for (int j = 1; j <= np; j++)
                    planet_kick(L, j, rx, ry, rz, ax, ay, az, flags, s_m, s_rh2, s_id);
            }
            r2 = fma(rx, rx, fma(ry, ry, rz * rz));
            if (lt_nonneg(r2, rh2_sun)) flags = 0x0001;
            if (gt_nonneg(r2, p.outer2)) flags = 0x0002;
            dti = first + s + 1;
            const double kc = (flags != 0 || dti == p.len) ? hdt : p.dt;
            vx = fma(ax, kc, vx);
            vy = fma(ay, kc, vy);
            vz = fma(az, kc, vz);
        }
        __syncthreads();
        if (tid == 0 && c + 2 < nchunks) {
            fence_proxy_async();
            issue_chunk(p, buf[b], &s_bar[b], c + 2, rec);
            pend[b] = (int)(c + 2);
        }
    }
    if (s_abort && tid == 0) {
        // drain the copies still in flight before the CTA's shared memory goes away
        for (int b = 0; b < 2; b++)
            if (pend[b] >= 0) (void)mbar_wait_bounded(&s_bar[b], ((uint32_t)pend[b] >> 1) & 1u);
    }

    if (active) {
        if (p.kill && (flags & 0x01)) flags = (uint16_t)((flags & 0xFF00) | 0x80);
        p.pa.rx[i] = rx; p.pa.ry[i] = ry; p.pa.rz[i] = rz;
        p.pa.vx[i] = vx; p.pa.vy[i] = vy; p.pa.vz[i] = vz;
        p.pa.ax[i] = ax; p.pa.ay[i] = ay; p.pa.az[i] = az;
        p.pa.flags[i] = flags;
        p.pa.deathtime_index[i] = dti;
    }

    // hand-off compaction: one atomic per warp
    const bool changed = active && flags != flags0;
    const unsigned lane = tid & 31u;
    const unsigned ballot = __ballot_sync(0xffffffffu, changed);
    if (ballot) {
        const unsigned leader = __ffs(ballot) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(p.ho.count, (uint32_t)__popc(ballot));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (changed) {
            uint32_t slot = base + __popc(ballot & ((1u << lane) - 1u));
            if (slot < p.ho.capacity) {
                p.ho.index[slot] = i;
                p.ho.id[slot] = p.pa.id[i];
                p.ho.flags[slot] = flags;
                p.ho.deathtime_index[slot] = dti;
            }
        }
    }
    if (p.ho.evals) {
        unsigned long long e = evals;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
        if (lane == 0 && e) atomicAdd(p.ho.evals, e);
    }
}

template <int NP>
cudaError_t launch_np(const KParams& p, size_t smem, cudaStream_t stream)
{
    auto kern = timeblock_kernel<NP>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    uint32_t grid = (p.n + BLOCK_THREADS - 1) / BLOCK_THREADS;
    kern<<<grid, BLOCK_THREADS, smem, stream>>>(p);
    return cudaGetLastError();
}

thread_local char g_err[256];

}  // namespace

size_t timeblock_smem_bytes(uint32_t npl, int chunk) { return 2ull * (size_t)chunk * 3u * npl * sizeof(double); }

const char* timeblock_error() { return g_err; }

int launch_timeblock(const glisser_particles* pa, size_t n_alive, const glisser_planet_block* pl,
                     const glisser_step_params* sp, const glisser_handoff* ho, cudaStream_t stream)
{
    if (!pa || !pl || !sp || !ho) return GLISSER_E_INVALID;
    if (pl->npl < 1 || pl->npl > (uint32_t)MAX_PLANETS) return GLISSER_E_INVALID;
    if (n_alive > 0xFFFFFFF0ull) return GLISSER_E_INVALID;
    if (!ho->count || !ho->status) return GLISSER_E_INVALID;
    if (ho->capacity && (!ho->index || !ho->id || !ho->flags || !ho->deathtime_index)) return GLISSER_E_INVALID;
    if (!(sp->dt > 0) || !(sp->outer_radius >= 0)) return GLISSER_E_INVALID;
    if (pl->len > 0) {
        if (!pl->log || !pl->m || !pl->id || !pl->rh) return GLISSER_E_INVALID;
        if (((uintptr_t)pl->log & 15u) != 0) return GLISSER_E_INVALID;
        if (pl->capacity < ((pl->len + 1u) & ~1u)) return GLISSER_E_INVALID;
    }
    if (n_alive == 0) return GLISSER_OK;

    KParams p;
    p.pa = *pa;
    p.n = (uint32_t)n_alive;
    p.log = pl->log;
    p.m = pl->m;
    p.pid = pl->id;
    p.rh = pl->rh;
    p.npl = pl->npl;
    p.len = pl->len;
    p.dt = sp->dt;
    p.outer2 = sp->outer_radius * sp->outer_radius;
    p.starter = sp->starter;
    p.kill = sp->kill_encounters;
    p.mlp = reinterpret_cast<const MlpDev*>(sp->mlp);
    if (p.starter == STARTER_LEARNED && !p.mlp) p.starter = STARTER_SERIES;
    p.ho = *ho;

    // chunk: as many steps as fit two buffers in 200 KB, at most LOG_CHUNK, even
    size_t rec_bytes = 3ull * pl->npl * sizeof(double);
    size_t fit = (200u * 1024u) / (2 * rec_bytes);
    uint32_t chunk = (uint32_t)(fit < (size_t)LOG_CHUNK ? fit : (size_t)LOG_CHUNK) & ~1u;
    if (chunk < 2) return GLISSER_E_INVALID;
    p.chunk = chunk;
    size_t smem = timeblock_smem_bytes(pl->npl, chunk);

    cudaError_t e;
    switch (pl->npl - 1) {
    case 0: e = launch_np<0>(p, smem, stream); break;
    case 1: e = launch_np<1>(p, smem, stream); break;
    case 2: e = launch_np<2>(p, smem, stream); break;
    case 3: e = launch_np<3>(p, smem, stream); break;
    case 4: e = launch_np<4>(p, smem, stream); break;
    case 5: e = launch_np<5>(p, smem, stream); break;
    case 6: e = launch_np<6>(p, smem, stream); break;
    case 7: e = launch_np<7>(p, smem, stream); break;
    case 8: e = launch_np<8>(p, smem, stream); break;
    default: e = launch_np<0>(p, smem, stream); break;
    }
    if (e != cudaSuccess) {
        snprintf(g_err, sizeof g_err, "time-block launch: %s", cudaGetErrorString(e));
        return GLISSER_E_CUDA;
    }
    return GLISSER_OK;
}

}  // namespace glisser
