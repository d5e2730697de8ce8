// Tile routine shared by the single-system and the ensemble time-block
// kernels (see timeblock.cu for the design).  Header-only: every function is
// device inline or host inline, compiled into each kernel translation unit.
#pragma once
#include "kepler.cuh"
#include "timeblock.cuh"

namespace glisser {
namespace tile {

struct Common {
    glisser_particles pa;
    uint32_t npl;
    uint32_t len;
    uint32_t chunk;
    double dt;
    double outer2;
    double tol_dt;          // Kepler residual tolerance x dt
    int starter;
    int kill;
    bool kick64;            // GLISSER_KICK_FP64: the FP64-kick kernels
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

// Bounded wait on an mbarrier phase: gives up after WAIT_NS of the global
// nanosecond timer (or WAIT_POLLS polls, whichever comes first) and returns
// false, so that a copy that never lands ends the kernel with a status bit
// instead of a hang.  A staged chunk normally lands in microseconds.
constexpr uint32_t WAIT_POLLS = 1u << 26;
constexpr uint64_t WAIT_NS = 2000000000ull;   // 2 s

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns = WAIT_NS)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t k = 0; k < WAIT_POLLS; k++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((k & 63u) == 0 && global_ns() - t0 > limit_ns) return false;
    }
    return false;
}

// Issues the copy of log chunk c into `buf`.  Bytes are rounded up to an
// even number of steps; the caller guarantees capacity for it.
__device__ __forceinline__ void issue_chunk(const Common& p, const double* log, double* buf, uint64_t* bar,
                                            uint32_t c, uint32_t rec)
{
    uint32_t first = c * p.chunk;
    uint32_t steps = min(p.chunk, p.len - first);
    steps = (steps + 1u) & ~1u;
    uint32_t bytes = steps * rec * 8u;
    mbar_expect_tx(bar, bytes);
    bulk_copy_g2s(buf, log + (size_t)first * rec, bytes, bar);
}

// What the float-float kick reads of planet j, packed in 32 bytes so that a
// step reads it with two 16-byte shared-memory loads instead of five.
struct __align__(16) PlanetConst {
    ff m;                       // m and rh^2 as float-floats
    ff rh2;
    double m15;                 // 1.5 m, the FP64 planet pull's form (its fallback)
    float rh2win;               // 2^-40 rh^2: the borderline window of the float-float radius test
    uint32_t id;
};

// Shared-memory state of one CTA.
struct CtaShared {
    double m[MAX_PLANETS];
    double rh2[MAX_PLANETS];
    uint32_t id[MAX_PLANETS];
    PlanetConst pk[MAX_PLANETS];
    uint64_t bar[2];
    int abort;
    uint32_t item;
};

// Threshold-borderline radius tests.  A flag is a discrete test of a squared
// distance against a squared radius (src/wh.cu:151, 163-169), so two correct
// evaluations that round differently can disagree for a particle sitting on
// the threshold.  Every test whose outcome counts is checked for a compared
// value within about 2^-40 (9e-13) of its threshold and counted: a zero count
// over a run shows that no flag of that run could depend on the rounding (the
// float-float kick's ~2^-48, or the last bits of an FP64 evaluation).
// near_nonneg: x within 2^13 units in the last place of t (x, t >= 0), on the
// integer pipe.
__device__ __forceinline__ uint32_t near_nonneg(double x, double t)
{
    const long long d = __double_as_longlong(x) - __double_as_longlong(t);
    return (unsigned long long)(d + 8192) <= 16384ull ? 1u : 0u;
}

// Pull of planet j, m dr / |dr|^3 with dr = r - r_j, added to the sum s,
// and its encounter test (src/wh.cu:145-160): the first planet inside its
// radius wins (flags == 0 guard).  All in float-float on the FP32 pipe (the
// position r and the staged planet log as float-floats): the planet terms
// are perturbations next to the Sun's pull, which the drift integrates in
// FP64, and carry ~1e-13 of their own size.
__device__ __forceinline__ void planet_kick(const ff* L, int j, ff rx, ff ry, ff rz, ff& sx, ff& sy, ff& sz,
                                            uint16_t& flags, uint32_t& border, const CtaShared& sh)
{
    const ff dx = ff_add(rx, ff_neg(L[3 * j]));
    const ff dy = ff_add(ry, ff_neg(L[3 * j + 1]));
    const ff dz = ff_add(rz, ff_neg(L[3 * j + 2]));
    const ff rad = ff_add(ff_add(ff_sqr(dx), ff_sqr(dy)), ff_sqr(dz));
    const PlanetConst q = sh.pk[j];
    if (flags == 0) {
        // rad.hi - rh2.hi is exact near the threshold (Sterbenz), so the FP32
        // difference is good to a few units of the low parts
        const float d = __fadd_rn(__fsub_rn(rad.hi, q.rh2.hi), __fsub_rn(rad.lo, q.rh2.lo));
        border += fabsf(d) <= q.rh2win ? 1u : 0u;
        if (ff_lt(rad, q.rh2)) flags = (uint16_t)((q.id << 8) | 0x0001);
    }
    const ff fac = pull_factor_ff(rad, q.m, q.m15);
    sx = ff_add(sx, ff_mul(dx, fac));
    sy = ff_add(sy, ff_mul(dy, fac));
    sz = ff_add(sz, ff_mul(dz, fac));
}

// The same kick term in FP64, as the reference computes it (src/wh.cu:142-160:
// the FP64 squared distance compared with the FP64 rh^2, a -= m dr / |dr|^3
// accumulated from a = h0), with |dr|^-3 from the FP64-accurate reciprocal
// square root (rsqrt_lean: within about one unit in the last place, the
// reference's 1 / (rad sqrt(rad)) to rounding).  The build's FP64-kick
// kernels use it (GLISSER_KICK_FP64).
__device__ __forceinline__ void planet_kick64(const double* L, int j, double rx, double ry, double rz, double& ax,
                                              double& ay, double& az, uint16_t& flags, uint32_t& border,
                                              const CtaShared& sh)
{
    const double dx = rx - L[3 * j], dy = ry - L[3 * j + 1], dz = rz - L[3 * j + 2];
    const double rad = fma(dx, dx, fma(dy, dy, dz * dz));
    if (flags == 0) {
        border += near_nonneg(rad, sh.rh2[j]);
        if (lt_nonneg(rad, sh.rh2[j])) flags = (uint16_t)((sh.id[j] << 8) | 0x0001);
    }
    const double y = rsqrt_lean(rad);
    const double fac = sh.m[j] * (y * (y * y));
    ax = fma(-dx, fac, ax);
    ay = fma(-dy, fac, ay);
    az = fma(-dz, fac, az);
}

// Integrates particles first + k*CTA + tid (k < PPT, below first + count)
// of one system over the block, staging that system's log through the two
// buffers.  `phase` counts completed waits per buffer (identical in every
// thread; carried across tiles of a persistent CTA).  Returns false after a
// staging timeout.  KICK64: the planet kick and its radius tests in FP64
// (planet_kick64) instead of float-float.
template <int NP, int CTA, int PPT, bool LEARNED, bool KICK64, int NET_ROWS = MLP_ROWS, int NET_QU = 1>
__device__ __forceinline__ bool run_tile(const Common& p, const double* log, uint32_t first, uint32_t count,
                                         double* stage, CtaShared& sh, uint32_t* phase)
{
    const int np = NP > 0 ? NP : (int)p.npl - 1;
    const uint32_t rec = 3u * (uint32_t)(np + 1);
    const size_t bufstride = (size_t)p.chunk * rec;
    const uint32_t tid = threadIdx.x;
    const uint32_t nchunks = (p.len + p.chunk - 1) / p.chunk;
    bool inflight0 = false, inflight1 = false;   // thread 0 only
    if (tid == 0) {
        if (nchunks > 0) { issue_chunk(p, log, stage, &sh.bar[0], 0, rec); inflight0 = true; }
        if (nchunks > 1) { issue_chunk(p, log, stage + bufstride, &sh.bar[1], 1, rec); inflight1 = true; }
    }

    // the acceleration is not carried between steps: each step's is used at
    // once for the merged kick, and the last one a particle reaches (flagged
    // or at the block's end) is stored at that step
    double rx[PPT], ry[PPT], rz[PPT], vx[PPT], vy[PPT], vz[PPT], r2[PPT], rinv[PPT];
    // neither the block-start flags nor the deathtime index are carried:
    // the index is stored at the particle's last step (flagged or the
    // block's end), and the start flags are read back from memory at the end
    uint16_t flags[PPT];
    uint32_t evals = 0, border = 0, nets = 0, wide = 0;
    const double hdt = p.dt * 0.5;
    const double mu = sh.m[0];
    const double rh2_sun = sh.rh2[0];
#pragma unroll
    for (int k = 0; k < PPT; k++) {
        const uint32_t off = (uint32_t)k * CTA + tid;
        const uint32_t i = first + off;
        rx[k] = ry[k] = rz[k] = vx[k] = vy[k] = vz[k] = 0;
        double a0x = 0, a0y = 0, a0z = 0;
        flags[k] = 0xFFFF;
        if (off < count) {
            rx[k] = p.pa.rx[i]; ry[k] = p.pa.ry[i]; rz[k] = p.pa.rz[i];
            vx[k] = p.pa.vx[i]; vy[k] = p.pa.vy[i]; vz[k] = p.pa.vz[i];
            a0x = p.pa.ax[i]; a0y = p.pa.ay[i]; a0z = p.pa.az[i];
            flags[k] = p.pa.flags[i];
        }
        // Kick-drift-kick with the two half kicks between consecutive steps
        // merged into one full kick (v += a dt); a particle takes the closing
        // half kick when it is flagged or the block ends, so its stored
        // velocity is always at a step boundary.  Each drift returns |r|^2 and
        // 1/|r| of the position it produces: the Sun/outer test's and the next
        // drift's.
        if (flags[k] == 0 && p.len > 0) {
            vx[k] = fma(a0x, hdt, vx[k]);
            vy[k] = fma(a0y, hdt, vy[k]);
            vz[k] = fma(a0z, hdt, vz[k]);
        }
        r2[k] = fma(rx[k], rx[k], fma(ry[k], ry[k], rz[k] * rz[k]));
        rinv[k] = rsqrt_lean(r2[k]);
    }

    bool ok = true;
    for (uint32_t c = 0; c < nchunks; c++) {
        const uint32_t b = c & 1u;
        if (!sh.abort) {
            if (!mbar_wait_bounded(&sh.bar[b], phase[b] & 1u)) {
                sh.abort = 1;
                atomicOr(p.ho.status, GLISSER_STATUS_LOG_TIMEOUT);
            }
        }
        __syncthreads();
        if (sh.abort) {
            ok = false;
            break;
        }
        phase[b]++;
        if (tid == 0) {
            if (b == 0) inflight0 = false;
            else inflight1 = false;
        }
        const uint32_t cfirst = c * p.chunk;
        const uint32_t steps = min(p.chunk, p.len - cfirst);
        double* Lw = stage + b * bufstride;
        if constexpr (!KICK64) {
            // the chunk's planet log as float-floats, in place (each 8-byte
            // double becomes the 8-byte pair of floats the kick reads)
            for (uint32_t i = tid; i < steps * rec; i += CTA) reinterpret_cast<ff*>(Lw)[i] = ff_split(Lw[i]);
        }
        __syncthreads();
        for (uint32_t s = 0; s < steps; s++) {
            const ff* L = reinterpret_cast<const ff*>(Lw) + (size_t)s * rec;
            const double* Ld = Lw + (size_t)s * rec;
#pragma unroll
            for (int k = 0; k < PPT; k++) {
                if (flags[k] != 0) continue;
                const DriftInvariants q =
                    drift_invariants(rx[k], ry[k], rz[k], vx[k], vy[k], vz[k], r2[k], rinv[k], p.dt, mu);
                DriftResult d = kepler_drift<LEARNED, NET_ROWS, NET_QU>(rx[k], ry[k], rz[k], vx[k], vy[k], vz[k], r2[k],
                                                                         rinv[k], q, p.dt, mu, p.starter, p.mlp,
                                                                         p.tol_dt);
                uint16_t fl = d.flags;
                evals += d.evals;
                if constexpr (LEARNED) nets += d.net;
                wide += d.wide;
                double aax, aay, aaz;
                if constexpr (KICK64) {
                    aax = Ld[0]; aay = Ld[1]; aaz = Ld[2];
                    if constexpr (NP > 0) {
#pragma unroll 1
                        for (int j = 1; j <= NP; j++)
                            planet_kick64(Ld, j, rx[k], ry[k], rz[k], aax, aay, aaz, fl, border, sh);
                    } else {
                        for (int j = 1; j <= np; j++)
                            planet_kick64(Ld, j, rx[k], ry[k], rz[k], aax, aay, aaz, fl, border, sh);
                    }
                } else {
                    const ff fx = ff_split(rx[k]), fy = ff_split(ry[k]), fz = ff_split(rz[k]);
                    ff sx = { 0.0f, 0.0f }, sy = { 0.0f, 0.0f }, sz = { 0.0f, 0.0f };
                    // the planet loop stays rolled: the kernel is bound by
                    // instruction fetch, and the unrolled four-planet
                    // float-float kick measured 9-12 % slower (the ensemble
                    // kernel and the single-system plain-giants kernel)
                    if constexpr (NP > 0) {
#pragma unroll 1
                        for (int j = 1; j <= NP; j++) planet_kick(L, j, fx, fy, fz, sx, sy, sz, fl, border, sh);
                    } else {
                        for (int j = 1; j <= np; j++) planet_kick(L, j, fx, fy, fz, sx, sy, sz, fl, border, sh);
                    }
                    // a = h0 - sum of the planets' pulls, to FP64 on the integer pipe
                    const ff gx = ff_add(L[0], ff_neg(sx)), gy = ff_add(L[1], ff_neg(sy)),
                             gz = ff_add(L[2], ff_neg(sz));
                    aax = ff_to_f64(gx);
                    aay = ff_to_f64(gy);
                    aaz = ff_to_f64(gz);
                }
                const double rr = r2[k];
                border += near_nonneg(rr, rh2_sun) + near_nonneg(rr, p.outer2);
                if (lt_nonneg(rr, rh2_sun)) fl = 0x0001;
                if (gt_nonneg(rr, p.outer2)) fl = 0x0002;
                flags[k] = fl;
                const uint32_t step = cfirst + s + 1;
                const bool last = fl != 0 || step == p.len;
                if (last) {
                    const uint32_t i = first + (uint32_t)k * CTA + tid;
                    p.pa.ax[i] = aax; p.pa.ay[i] = aay; p.pa.az[i] = aaz;
                    p.pa.deathtime_index[i] = step;
                }
                const double kc = last ? hdt : p.dt;
                vx[k] = fma(aax, kc, vx[k]);
                vy[k] = fma(aay, kc, vy[k]);
                vz[k] = fma(aaz, kc, vz[k]);
            }
        }
        __syncthreads();
        if (tid == 0 && c + 2 < nchunks) {
            fence_proxy_async();
            issue_chunk(p, log, stage + b * bufstride, &sh.bar[b], c + 2, rec);
            if (b == 0) inflight0 = true;
            else inflight1 = true;
        }
    }
    if (!ok && tid == 0) {
        // drain the copies still in flight before the shared memory is reused or released
        if (inflight0) (void)mbar_wait_bounded(&sh.bar[0], phase[0] & 1u);
        if (inflight1) (void)mbar_wait_bounded(&sh.bar[1], phase[1] & 1u);
    }

    const unsigned lane = tid & 31u;
#pragma unroll
    for (int k = 0; k < PPT; k++) {
        const uint32_t off = (uint32_t)k * CTA + tid;
        const uint32_t i = first + off;
        const bool active = off < count;
        uint16_t flags0 = 0xFFFF;
        bool ran = false;
        if (active) {
            flags0 = p.pa.flags[i];         // the block-start flags, not yet overwritten
            // integrated: its deathtime index was stored at its last step
            ran = flags0 == 0 && p.len > 0;
            if (p.kill == GLISSER_ENCOUNTERS_KILL && (flags[k] & 0x01))
                flags[k] = (uint16_t)((flags[k] & 0xFF00) | 0x80);
            // a rolled-back encounter particle leaves its block-start state in
            // place (nothing has overwritten it yet)
            const bool rollback =
                p.kill == GLISSER_ENCOUNTERS_ROLLBACK && flags[k] != 0 && (flags[k] & 0xFE) == 0;
            if (!rollback) {
                p.pa.rx[i] = rx[k]; p.pa.ry[i] = ry[k]; p.pa.rz[i] = rz[k];
                p.pa.vx[i] = vx[k]; p.pa.vy[i] = vy[k]; p.pa.vz[i] = vz[k];
            }
            p.pa.flags[i] = flags[k];
            if (!ran) p.pa.deathtime_index[i] = 0;
        }
        // hand-off compaction: one atomic per warp
        const bool changed = active && flags[k] != flags0;
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
                    p.ho.flags[slot] = flags[k];
                    p.ho.deathtime_index[slot] = ran ? p.pa.deathtime_index[i] : 0u;
                }
            }
        }
    }
    if (p.ho.evals) {
        unsigned long long e = evals;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
        if (lane == 0 && e) atomicAdd(p.ho.evals, e);
    }
    if (p.ho.borderline) {
        unsigned long long e = border;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
        if (lane == 0 && e) atomicAdd(p.ho.borderline, e);
    }
    if (p.ho.wide) {
        unsigned long long e = wide;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
        if (lane == 0 && e) atomicAdd(p.ho.wide, e);
    }
    if constexpr (LEARNED) {
        if (p.ho.learned) {
            unsigned long long e = nets;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
            if (lane == 0 && e) atomicAdd(p.ho.learned, e);
        }
    }
    return ok;
}

__device__ __forceinline__ void load_planet_constants(CtaShared& sh, uint32_t npl, const double* m, const double* rh,
                                                      const uint32_t* pid)
{
    for (uint32_t j = threadIdx.x; j < npl; j += blockDim.x) {
        sh.m[j] = m[j];
        sh.rh2[j] = rh[j] * rh[j];
        sh.id[j] = pid[j];
        PlanetConst q;
        q.m = ff_split(m[j]);
        q.rh2 = ff_split(sh.rh2[j]);
        q.m15 = 1.5 * m[j];
        q.rh2win = q.rh2.hi * 0x1p-40f;
        q.id = pid[j];
        sh.pk[j] = q;
    }
}

__device__ __forceinline__ void init_barriers(CtaShared& sh)
{
    if (threadIdx.x == 0) {
        sh.abort = 0;
        mbar_init(&sh.bar[0], 1);
        mbar_init(&sh.bar[1], 1);
        mbar_fence_init();
    }
}


inline bool fill_common(Common& p, const glisser_particles* pa, const glisser_step_params* sp, const glisser_handoff* ho,
                 uint32_t npl, uint32_t len, uint32_t max_chunk = LOG_CHUNK)
{
    p.pa = *pa;
    p.npl = npl;
    p.len = len;
    p.dt = sp->dt;
    p.outer2 = sp->outer_radius * sp->outer_radius;
    p.tol_dt = (sp->kepler_tol > 0 ? sp->kepler_tol : KEP_TOL) * sp->dt;
    p.starter = sp->starter;
    p.kill = sp->kill_encounters;
    p.kick64 = sp->kick == GLISSER_KICK_FP64;
    p.mlp = reinterpret_cast<const MlpDev*>(sp->mlp);
    if (p.starter == STARTER_LEARNED && !p.mlp) p.starter = STARTER_SERIES;
    p.ho = *ho;
    p.chunk = log_chunk_steps(npl, max_chunk);
    return p.chunk >= 2;
}

inline bool handoff_ok(const glisser_handoff* ho)
{
    if (!ho->count || !ho->status) return false;
    return !(ho->capacity && (!ho->index || !ho->id || !ho->flags || !ho->deathtime_index));
}

}  // namespace tile
}  // namespace glisser
