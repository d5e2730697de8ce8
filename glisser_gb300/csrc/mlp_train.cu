// Learned Kepler starter: logging of plain-method solves, training on the GPU
// with hand-written forward/backward kernels (BF16 weights in, FP32
// accumulation), and the device copy of the weights the drift reads.
//
// Training kernel layout: one CTA of 128 threads takes a tile of 128
// samples, one per thread.  Each thread runs the forward pass of its sample
// in the order of mlp_forward, the inputs and the hidden activations rounded
// to the BF16 hi + lo pairs its products read (gradients straight through
// the rounding), so the trained network is the one the drift evaluates; it
// keeps the pre-activations of the second layer in registers, and runs the backward pass to the per-sample deltas, which it
// writes to shared-memory tiles (rows padded to 33 floats: the row-per-thread
// writes and the column reads are both bank-conflict free).  The weight
// gradients are then sums over the tile's samples -- the FP32-accumulated
// products of the stored activations and deltas -- computed with each thread
// owning a fixed set of parameters, and written as one partial per CTA.  A
// second kernel sums the partials in a fixed order (deterministic) and takes
// the Adam step on the FP32 master weights; the next forward pass re-rounds
// them to BF16.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "kepler.cuh"
#include "mlp_train.h"

namespace glisser {

namespace {

constexpr int TT = 128;                  // samples per training tile (one per thread)
constexpr int HP = MLP_H + 1;            // padded activation row
constexpr int PART = MLP_NPARAM + 1;     // per-CTA partial: gradients, then the loss sum
constexpr int SM_WEIGHTS = MLP_H * 4 + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 4;
constexpr int SM_FLOATS = SM_WEIGHTS + 4 * TT * HP + TT * 4 + 2 * TT;

void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

__device__ __forceinline__ uint32_t mix32(uint64_t x)
{
    // splitmix64 finaliser
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (uint32_t)(x >> 32);
}

// One plain-method solve per state (classic starter, quartic Newton, Laguerre
// fallback: the drift's own solver) with the invariants computed exactly as
// the drift computes them.  Non-converged solves get a NaN target, which the
// training kernel skips.  Only solves with f0 >= f0_min count towards
// evals_sum (the ones the host keeps).
__global__ void log_solves_kernel(glisser_particles pa, uint32_t n, double dt, double mu, float* feat, float* target,
                                  unsigned long long* evals_sum, float f0_min)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t evals = 0;
    if (i < n) {
        const double rx = pa.rx[i], ry = pa.ry[i], rz = pa.rz[i];
        const double vx = pa.vx[i], vy = pa.vy[i], vz = pa.vz[i];
        const double r2 = fma(rx, rx, fma(ry, ry, rz * rz));
        const double v2 = fma(vx, vx, fma(vy, vy, vz * vz));
        const double u = fma(rx, vx, fma(ry, vy, rz * vz));
        const double rinv = rsqrt_lean(r2);
        const double r0 = r2 * rinv;
        const double mu_r = mu * rinv;
        const double alpha = fma(2.0, mu_r, -v2);
        const double dt2mu = dt * dt * mu;
        const double tau2 = dt2mu * (rinv * rinv) * rinv;
        double s = starter_classic(dt, r0, rinv, mu, alpha, u);
        const double tol = KEP_TOL * dt;
        GFun g;
        double ds = 0;
        uint16_t ev = 0;
        bool ok = kepler_newton(s, dt, r0, u, mu, alpha, tol, tau2_f32(dt * rinv, mu_r) < SMALL_STEP_TAU2, g, ds, ev);
        if (!ok) ok = kepler_laguerre(s, dt, r0, u, mu, alpha, tol, g, ds, ev);
        float f0, f1, f2;
        mlp_features(tau2_f32(dt * rinv, mu_r), u, rinv, mu_r, alpha, f0, f1, f2);
        evals = f0 >= f0_min ? ev : 0u;
        const double sf = s + ds;
        feat[3 * (size_t)i] = f0;
        feat[3 * (size_t)i + 1] = f1;
        feat[3 * (size_t)i + 2] = f2;
        target[i] = (ok && sf > 0) ? (float)(log(sf * r0 / dt) / sqrt(tau2)) : __int_as_float(0x7fc00000);
    }
    unsigned long long e = evals;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    if ((threadIdx.x & 31u) == 0 && e) atomicAdd(evals_sum, e);
}

struct TrainArgs {
    const float* feat;
    const float* target;
    uint32_t n;            // samples in the data set
    uint32_t batch;        // samples in this minibatch
    uint32_t sequential;   // 1: sample = global thread index; 0: seeded draw with replacement
    uint32_t step;
    uint64_t seed;
    float inv_batch;
    MlpNorm norm;
};

__device__ __forceinline__ float dsilu(float a)
{
    const float s = mlp_sigmoid(a);
    return s * fmaf(a, 1.0f - s, 1.0f);
}

__global__ void __launch_bounds__(TT) grad_kernel(const float* __restrict__ params, const TrainArgs a,
                                                  float* __restrict__ partials)
{
    extern __shared__ float sm[];
    float* W1 = sm;                       // [MLP_H][4]
    float* B1 = W1 + MLP_H * 4;
    float* W2 = B1 + MLP_H;               // [MLP_H][MLP_H]
    float* B2 = W2 + MLP_H * MLP_H;
    float* W3 = B2 + MLP_H;
    float* B3 = W3 + MLP_H;               // [4]
    float* H1 = B3 + 4;                   // [TT][HP] layer-1 activations
    float* H2 = H1 + TT * HP;             // layer-2 activations
    float* D1 = H2 + TT * HP;             // layer-1 pre-activation deltas
    float* D2 = D1 + TT * HP;             // layer-2 pre-activation deltas
    float* X = D2 + TT * HP;              // [TT][4] normalised inputs
    float* DY = X + TT * 4;               // [TT] output deltas
    float* LS = DY + TT;                  // [TT] squared errors

    const int t = threadIdx.x;
    for (int q = t; q < MLP_H * 4; q += TT) {
        const int j = q >> 2, k = q & 3;
        W1[q] = k < MLP_IN ? bf16_round(params[MLP_OFF_W1 + j * MLP_IN + k]) : 0.0f;
    }
    for (int q = t; q < MLP_H * MLP_H; q += TT) W2[q] = bf16_round(params[MLP_OFF_W2 + q]);
    if (t < MLP_H) {
        B1[t] = params[MLP_OFF_B1 + t];
        B2[t] = params[MLP_OFF_B2 + t];
        W3[t] = bf16_round(params[MLP_OFF_W3 + t]);
    }
    if (t == 0) B3[0] = params[MLP_OFF_B3];
    __syncthreads();

    // this thread's sample
    const uint32_t gi = blockIdx.x * TT + t;
    bool valid = gi < a.batch;
    float f0 = 0, f1 = 0, f2 = 0, tg = 0;
    if (valid) {
        const uint32_t idx = a.sequential ? gi : mix32(a.seed ^ ((uint64_t)a.step << 32) ^ gi) % a.n;
        f0 = a.feat[3 * (size_t)idx];
        f1 = a.feat[3 * (size_t)idx + 1];
        f2 = a.feat[3 * (size_t)idx + 2];
        tg = a.target[idx];
        valid = isfinite(tg) && isfinite(f0) && isfinite(f1) && isfinite(f2);
    }
    float x0 = 0, x1 = 0, x2 = 0, tn = 0;
    if (valid) {
        // the inputs as the first layer reads them (BF16 hi + lo)
        x0 = bf16_split_sum((f0 - a.norm.in_mean[0]) * a.norm.in_scale[0]);
        x1 = bf16_split_sum((f1 - a.norm.in_mean[1]) * a.norm.in_scale[1]);
        x2 = bf16_split_sum((f2 - a.norm.in_mean[2]) * a.norm.in_scale[2]);
        tn = (tg - a.norm.out_mean) / a.norm.out_scale;
    }

    // forward, in the order of mlp_forward
    float* h1 = H1 + t * HP;
    float* h2 = H2 + t * HP;
#pragma unroll 4
    for (int j = 0; j < MLP_H; j++) {
        float z = B1[j];
        z = fmaf(W1[4 * j], x0, z);
        z = fmaf(W1[4 * j + 1], x1, z);
        z = fmaf(W1[4 * j + 2], x2, z);
        h1[j] = bf16_split_sum(z * mlp_sigmoid(z));   // as the hidden layer reads it; straight-through below
    }
    float a2[MLP_H];
    float y = B3[0];
#pragma unroll
    for (int j = 0; j < MLP_H; j++) {
        float z = B2[j];
#pragma unroll
        for (int k = 0; k < MLP_H; k++) z = fmaf(W2[j * MLP_H + k], h1[k], z);
        a2[j] = z;
        const float hv = z * mlp_sigmoid(z);
        h2[j] = hv;
        y = fmaf(W3[j], hv, y);
    }
    const float err = valid ? y - tn : 0.0f;
    const float dy = 2.0f * err * a.inv_batch;
    LS[t] = err * err;
    DY[t] = dy;
    X[4 * t] = x0;
    X[4 * t + 1] = x1;
    X[4 * t + 2] = x2;

    // backward to the per-sample deltas
    float* d2 = D2 + t * HP;
    float* d1 = D1 + t * HP;
#pragma unroll
    for (int j = 0; j < MLP_H; j++) d2[j] = dy * W3[j] * dsilu(a2[j]);
#pragma unroll 4
    for (int k = 0; k < MLP_H; k++) {
        float z = B1[k];
        z = fmaf(W1[4 * k], x0, z);
        z = fmaf(W1[4 * k + 1], x1, z);
        z = fmaf(W1[4 * k + 2], x2, z);
        float dh = 0.0f;
#pragma unroll 8
        for (int j = 0; j < MLP_H; j++) dh = fmaf(W2[j * MLP_H + k], d2[j], dh);
        d1[k] = dh * dsilu(z);
    }
    __syncthreads();

    // parameter gradients summed over the tile
    float* out = partials + (size_t)blockIdx.x * PART;
    {
        // W2: thread t owns row j = t / 4, columns 8 (t % 4) .. + 7
        const int j = t >> 2, kb = (t & 3) * 8;
        float acc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
        for (int i = 0; i < TT; i++) {
            const float d = D2[i * HP + j];
#pragma unroll
            for (int q = 0; q < 8; q++) acc[q] = fmaf(d, H1[i * HP + kb + q], acc[q]);
        }
#pragma unroll
        for (int q = 0; q < 8; q++) out[MLP_OFF_W2 + j * MLP_H + kb + q] = acc[q];
    }
    if (t < MLP_H * MLP_IN) {
        const int j = t / MLP_IN, k = t % MLP_IN;
        float acc = 0;
        for (int i = 0; i < TT; i++) acc = fmaf(D1[i * HP + j], X[4 * i + k], acc);
        out[MLP_OFF_W1 + t] = acc;
    } else {
        const int j = t - MLP_H * MLP_IN;
        float acc = 0;
        for (int i = 0; i < TT; i++) acc += D1[i * HP + j];
        out[MLP_OFF_B1 + j] = acc;
    }
    if (t < MLP_H) {
        float acc = 0;
        for (int i = 0; i < TT; i++) acc += D2[i * HP + t];
        out[MLP_OFF_B2 + t] = acc;
    } else if (t < 2 * MLP_H) {
        const int j = t - MLP_H;
        float acc = 0;
        for (int i = 0; i < TT; i++) acc = fmaf(DY[i], H2[i * HP + j], acc);
        out[MLP_OFF_W3 + j] = acc;
    } else if (t == 2 * MLP_H) {
        float acc = 0;
        for (int i = 0; i < TT; i++) acc += DY[i];
        out[MLP_OFF_B3] = acc;
    } else if (t == 2 * MLP_H + 1) {
        float acc = 0;
        for (int i = 0; i < TT; i++) acc += LS[i];
        out[MLP_NPARAM] = acc;
    }
}

struct AdamArgs {
    float lr, b1, b2, eps, bc1, bc2, inv_batch;
    uint32_t apply;        // 0: only sum the partials into `grad`
};

// Sums the CTA partials in CTA order; then (apply) one Adam step.  grad
// (optional) receives the summed gradients and, at index MLP_NPARAM, the
// mean loss.
__global__ void adam_kernel(float* params, float* m, float* v, const float* __restrict__ partials, uint32_t nblk,
                            AdamArgs a, float* grad)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > (uint32_t)MLP_NPARAM) return;
    float g = 0;
    for (uint32_t b = 0; b < nblk; b++) g += partials[(size_t)b * PART + p];
    if (p == (uint32_t)MLP_NPARAM) {
        if (grad) grad[p] = g * a.inv_batch;
        return;
    }
    if (grad) grad[p] = g;
    if (!a.apply) return;
    const float mm = fmaf(a.b1, m[p] - g, g);          // b1 m + (1 - b1) g
    const float vv = fmaf(a.b2, v[p] - g * g, g * g);
    m[p] = mm;
    v[p] = vv;
    params[p] -= a.lr * (mm / a.bc1) / (sqrtf(vv / a.bc2) + a.eps);
}

// The time-block kernels' inference (mlp_forward) over a feature list (NaN
// outside the box).
__global__ void __launch_bounds__(128) predict_kernel(const MlpDev* __restrict__ w, const float* __restrict__ feat,
                                                      uint32_t n, float* y)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const MlpNorm& nm = w->norm;
    const float f0 = feat[3 * (size_t)i], f1 = feat[3 * (size_t)i + 1], f2 = feat[3 * (size_t)i + 2];
    const bool in_box = f0 >= nm.x_lo[0] && f0 <= nm.x_hi[0] && f1 >= nm.x_lo[1] && f1 <= nm.x_hi[1] &&
                        f2 >= nm.x_lo[2] && f2 <= nm.x_hi[2];
    if (!in_box) {
        y[i] = __int_as_float(0x7fc00000);
        return;
    }
    const float out = mlp_forward(w, (f0 - nm.in_mean[0]) * nm.in_scale[0], (f1 - nm.in_mean[1]) * nm.in_scale[1],
                                  (f2 - nm.in_mean[2]) * nm.in_scale[2]);
    y[i] = fmaf(nm.out_scale, out, nm.out_mean);
}

// One Kepler drift per state with the time-block kernel's drift routine.
template <bool LEARNED>
__global__ void drift_states_kernel(glisser_particles pa, uint32_t n, double dt, double mu, int starter,
                                    const MlpDev* mlp, uint32_t* evals, uint16_t* flags)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double rx = pa.rx[i], ry = pa.ry[i], rz = pa.rz[i], vx = pa.vx[i], vy = pa.vy[i], vz = pa.vz[i];
    const double r2 = fma(rx, rx, fma(ry, ry, rz * rz));
    double r2v = r2, rinv = rsqrt_lean(r2);
    DriftResult d = kepler_drift<LEARNED>(rx, ry, rz, vx, vy, vz, r2v, rinv, dt, mu, starter, mlp, KEP_TOL * dt);
    pa.rx[i] = rx; pa.ry[i] = ry; pa.rz[i] = rz;
    pa.vx[i] = vx; pa.vy[i] = vy; pa.vz[i] = vz;
    if (evals) evals[i] = d.evals;
    if (flags) flags[i] = d.flags;
}

uint32_t bf16_bits_round(float x)
{
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);   // round to nearest even (finite values)
    return u & 0xFFFF0000u;
}

float bf16_round_host(float x)
{
    if (!std::isfinite(x)) return x;
    uint32_t u = bf16_bits_round(x);
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

bool is_weight(int p)
{
    return (p >= MLP_OFF_W1 && p < MLP_OFF_B1) || (p >= MLP_OFF_W2 && p < MLP_OFF_B2) ||
           (p >= MLP_OFF_W3 && p < MLP_OFF_B3);
}

MlpDev make_dev(const float* params, const MlpNorm& norm)
{
    MlpDev d;
    std::memset(&d, 0, sizeof d);
    for (int j = 0; j < MLP_H; j++) {
        for (int k = 0; k < MLP_IN; k++) d.w1[j][k] = bf16_round_host(params[MLP_OFF_W1 + j * MLP_IN + k]);
        d.b1[j] = params[MLP_OFF_B1 + j];
        for (int k = 0; k < MLP_H; k++) d.w2[j][k] = bf16_round_host(params[MLP_OFF_W2 + j * MLP_H + k]);
        d.b2[j] = params[MLP_OFF_B2 + j];
        d.w3[j] = bf16_round_host(params[MLP_OFF_W3 + j]);
    }
    d.b3 = params[MLP_OFF_B3];
    d.norm = norm;
    return d;
}

}  // namespace

void* mlp_upload(const std::vector<uint8_t>& file)
{
    if (file.size() != sizeof(MlpFileHeader) + MLP_NPARAM * sizeof(float))
        throw std::invalid_argument("learned-starter weights file has the wrong size");
    MlpFileHeader h;
    std::memcpy(&h, file.data(), sizeof h);
    if (std::memcmp(h.magic, "GLMLP001", 8) != 0 || h.nparam != (uint32_t)MLP_NPARAM || h.hidden != (uint32_t)MLP_H)
        throw std::invalid_argument("not a learned-starter weights file (magic GLMLP001, 3-32-32-1)");
    std::vector<float> params(MLP_NPARAM);
    std::memcpy(params.data(), file.data() + sizeof h, MLP_NPARAM * sizeof(float));
    MlpDev dev = make_dev(params.data(), h.norm);
    void* d = nullptr;
    if (cudaMalloc(&d, sizeof(MlpDev)) != cudaSuccess) throw std::bad_alloc();
    if (cudaMemcpy(d, &dev, sizeof dev, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        throw std::runtime_error("learned-starter weights upload failed");
    }
    return d;
}

void mlp_free(void* d)
{
    if (d) cudaFree(d);
}

MlpTrainer::MlpTrainer(size_t capacity, uint64_t seed) : cap_(capacity), params_(MLP_NPARAM, 0.0f)
{
    if (capacity == 0 || capacity > 0xFFFFFFF0ull) throw std::invalid_argument("sample capacity out of range");
    std::memset(&norm, 0, sizeof norm);
    for (int k = 0; k < 4; k++) {
        norm.in_scale[k] = 1.0f;
        norm.x_lo[k] = -INFINITY;
        norm.x_hi[k] = INFINITY;
    }
    norm.out_scale = 1.0f;
    // He-uniform initial weights (bound sqrt(6 / fan_in)), zero biases
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int count, int fan_in) {
        std::uniform_real_distribution<float> u(-std::sqrt(6.0f / fan_in), std::sqrt(6.0f / fan_in));
        for (int q = 0; q < count; q++) params_[off + q] = u(rng);
    };
    fill(MLP_OFF_W1, MLP_H * MLP_IN, MLP_IN);
    fill(MLP_OFF_W2, MLP_H * MLP_H, MLP_H);
    fill(MLP_OFF_W3, MLP_H, MLP_H);
    check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
    check(cudaMalloc(&d_feat_, cap_ * 3 * sizeof(float)), "sample buffer");
    check(cudaMalloc(&d_target_, cap_ * sizeof(float)), "sample buffer");
    check(cudaMalloc(&d_params_, MLP_NPARAM * sizeof(float)), "parameters");
    check(cudaMalloc(&d_m_, MLP_NPARAM * sizeof(float)), "Adam state");
    check(cudaMalloc(&d_v_, MLP_NPARAM * sizeof(float)), "Adam state");
    check(cudaMalloc(&d_loss_, (MLP_NPARAM + 1) * sizeof(float)), "loss");
    check(cudaMalloc(&d_evals_, sizeof(unsigned long long)), "counter");
    check(cudaMalloc(&d_dev_, sizeof(MlpDev)), "weights");
    check(cudaMemset(d_m_, 0, MLP_NPARAM * sizeof(float)), "memset");
    check(cudaMemset(d_v_, 0, MLP_NPARAM * sizeof(float)), "memset");
    check(cudaMemset(d_evals_, 0, sizeof(unsigned long long)), "memset");
    check(cudaMemcpy(d_params_, params_.data(), MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice), "upload");
    check(cudaFuncSetAttribute(grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(SM_FLOATS * sizeof(float))),
          "grad kernel attribute");
}

MlpTrainer::~MlpTrainer()
{
    cudaFree(d_feat_); cudaFree(d_target_); cudaFree(d_params_); cudaFree(d_m_); cudaFree(d_v_);
    cudaFree(d_partials_); cudaFree(d_loss_); cudaFree(d_evals_); cudaFree(d_dev_);
    if (stream_) cudaStreamDestroy(stream_);
}

size_t MlpTrainer::log_states(const glisser_particles& pa, size_t n, double dt, double mu, cudaStream_t stream)
{
    size_t m = std::min(n, cap_ - n_);
    if (m == 0) return 0;
    glisser_particles p = pa;
    // f0 = log(tau) >= log(tau2_min) / 2
    const float f0_min = log_tau2_min_ > 0 ? (float)(0.5 * std::log(log_tau2_min_)) : -INFINITY;
    log_solves_kernel<<<(unsigned)((m + 255) / 256), 256, 0, stream>>>(p, (uint32_t)m, dt, mu, d_feat_ + 3 * n_,
                                                                        d_target_ + n_, d_evals_, f0_min);
    check(cudaGetLastError(), "log_solves_kernel");
    check(cudaStreamSynchronize(stream), "log_solves_kernel");
    if (log_tau2_min_ > 0) {
        // keep the solves at or above the floor, in their order
        std::vector<float> f(3 * m), y(m);
        check(cudaMemcpy(f.data(), d_feat_ + 3 * n_, f.size() * sizeof(float), cudaMemcpyDeviceToHost), "samples");
        check(cudaMemcpy(y.data(), d_target_ + n_, y.size() * sizeof(float), cudaMemcpyDeviceToHost), "samples");
        size_t k = 0;
        for (size_t i = 0; i < m; i++) {
            if (!(f[3 * i] >= f0_min)) continue;
            f[3 * k] = f[3 * i];
            f[3 * k + 1] = f[3 * i + 1];
            f[3 * k + 2] = f[3 * i + 2];
            y[k] = y[i];
            k++;
        }
        if (k > 0) {
            check(cudaMemcpy(d_feat_ + 3 * n_, f.data(), 3 * k * sizeof(float), cudaMemcpyHostToDevice), "samples");
            check(cudaMemcpy(d_target_ + n_, y.data(), k * sizeof(float), cudaMemcpyHostToDevice), "samples");
        }
        m = k;
    }
    n_ += m;
    return m;
}

void MlpTrainer::add_samples(const float* feat, const float* target, size_t n)
{
    size_t m = std::min(n, cap_ - n_);
    check(cudaMemcpy(d_feat_ + 3 * n_, feat, m * 3 * sizeof(float), cudaMemcpyHostToDevice), "samples");
    check(cudaMemcpy(d_target_ + n_, target, m * sizeof(float), cudaMemcpyHostToDevice), "samples");
    n_ += m;
}

void MlpTrainer::get_samples(float* feat, float* target, size_t first, size_t n) const
{
    if (first > n_ || n > n_ - first) throw std::invalid_argument("get_samples: range beyond the logged samples");
    if (n == 0) return;
    if (feat) check(cudaMemcpy(feat, d_feat_ + 3 * first, n * 3 * sizeof(float), cudaMemcpyDeviceToHost), "samples");
    if (target) check(cudaMemcpy(target, d_target_ + first, n * sizeof(float), cudaMemcpyDeviceToHost), "samples");
}

unsigned long long MlpTrainer::plain_evals()
{
    unsigned long long e = 0;
    check(cudaMemcpy(&e, d_evals_, sizeof e, cudaMemcpyDeviceToHost), "counter");
    return e;
}

void MlpTrainer::fit_norm()
{
    if (n_ == 0) throw std::invalid_argument("no samples logged");
    std::vector<float> f(n_ * 3), y(n_);
    check(cudaMemcpy(f.data(), d_feat_, f.size() * sizeof(float), cudaMemcpyDeviceToHost), "samples");
    check(cudaMemcpy(y.data(), d_target_, y.size() * sizeof(float), cudaMemcpyDeviceToHost), "samples");
    double s[3] = { 0, 0, 0 }, s2[3] = { 0, 0, 0 }, ys = 0, ys2 = 0;
    float lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    size_t cnt = 0;
    for (size_t i = 0; i < n_; i++) {
        const float* fi = &f[3 * i];
        if (!std::isfinite(y[i]) || !std::isfinite(fi[0]) || !std::isfinite(fi[1]) || !std::isfinite(fi[2])) continue;
        for (int k = 0; k < 3; k++) {
            s[k] += fi[k];
            s2[k] += (double)fi[k] * fi[k];
            lo[k] = std::min(lo[k], fi[k]);
            hi[k] = std::max(hi[k], fi[k]);
        }
        ys += y[i];
        ys2 += (double)y[i] * y[i];
        cnt++;
    }
    if (cnt < 2) throw std::invalid_argument("fewer than two usable samples");
    for (int k = 0; k < 3; k++) {
        double mean = s[k] / cnt, var = std::max(s2[k] / cnt - mean * mean, 1e-30);
        norm.in_mean[k] = (float)mean;
        norm.in_scale[k] = (float)(1.0 / std::sqrt(var));
        norm.x_lo[k] = lo[k];
        norm.x_hi[k] = hi[k];
    }
    norm.in_mean[3] = 0;
    norm.in_scale[3] = 1;
    norm.x_lo[3] = norm.x_hi[3] = 0;
    double ym = ys / cnt, yv = std::max(ys2 / cnt - ym * ym, 1e-30);
    norm.out_mean = (float)ym;
    norm.out_scale = (float)std::sqrt(yv);
    norm_set = true;
    dev_stale_ = true;
}

void MlpTrainer::get_params(float* out) const { std::memcpy(out, params_.data(), MLP_NPARAM * sizeof(float)); }

void MlpTrainer::set_params(const float* in)
{
    std::memcpy(params_.data(), in, MLP_NPARAM * sizeof(float));
    check(cudaMemcpy(d_params_, params_.data(), MLP_NPARAM * sizeof(float), cudaMemcpyHostToDevice), "upload");
    check(cudaMemset(d_m_, 0, MLP_NPARAM * sizeof(float)), "memset");
    check(cudaMemset(d_v_, 0, MLP_NPARAM * sizeof(float)), "memset");
    adam_t_ = 0;
    dev_stale_ = true;
}

void MlpTrainer::ensure_partials(size_t blocks)
{
    if (blocks <= partials_cap_) return;
    cudaFree(d_partials_);
    d_partials_ = nullptr;
    check(cudaMalloc(&d_partials_, blocks * PART * sizeof(float)), "partials");
    partials_cap_ = blocks;
}

void MlpTrainer::grad_launch(const float* feat, const float* target, uint32_t n, uint32_t batch, bool sequential,
                             uint64_t seed, uint32_t step, uint32_t blocks)
{
    TrainArgs a;
    a.feat = feat;
    a.target = target;
    a.n = n;
    a.batch = batch;
    a.sequential = sequential ? 1u : 0u;
    a.step = step;
    a.seed = seed;
    a.inv_batch = 1.0f / (float)batch;
    a.norm = norm;
    grad_kernel<<<blocks, TT, SM_FLOATS * sizeof(float), stream_>>>(d_params_, a, d_partials_);
    check(cudaGetLastError(), "grad_kernel");
}

void MlpTrainer::train(int steps, int batch, float lr, float lr_min, uint64_t seed, float* losses)
{
    if (n_ == 0 || !norm_set) throw std::invalid_argument("train: log samples and fit the normalisation first");
    if (steps < 0 || batch < TT || batch % TT != 0) throw std::invalid_argument("train: batch must be a multiple of 128");
    const uint32_t blocks = (uint32_t)(batch / TT);
    ensure_partials(blocks);
    std::vector<float> hl(losses ? steps : 0);
    const float b1 = 0.9f, b2 = 0.999f;
    for (int s = 0; s < steps; s++) {
        grad_launch(d_feat_, d_target_, (uint32_t)n_, (uint32_t)batch, false, seed, (uint32_t)s, blocks);
        adam_t_++;
        const double c = 0.5 * (1.0 + std::cos(3.14159265358979323846 * (double)s / std::max(1, steps)));
        AdamArgs a;
        a.lr = (float)(lr_min + (lr - lr_min) * c);
        a.b1 = b1;
        a.b2 = b2;
        a.eps = 1e-8f;
        a.bc1 = (float)(1.0 - std::pow((double)b1, adam_t_));
        a.bc2 = (float)(1.0 - std::pow((double)b2, adam_t_));
        a.inv_batch = 1.0f / (float)batch;
        a.apply = 1;
        adam_kernel<<<(MLP_NPARAM + 1 + 127) / 128, 128, 0, stream_>>>(d_params_, d_m_, d_v_, d_partials_, blocks, a,
                                                                      losses ? d_loss_ : nullptr);
        check(cudaGetLastError(), "adam_kernel");
        if (losses) {
            check(cudaMemcpyAsync(&hl[s], d_loss_ + MLP_NPARAM, sizeof(float), cudaMemcpyDeviceToHost, stream_), "loss");
        }
    }
    check(cudaStreamSynchronize(stream_), "training");
    if (losses) std::memcpy(losses, hl.data(), steps * sizeof(float));
    check(cudaMemcpy(params_.data(), d_params_, MLP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost), "parameters");
    dev_stale_ = true;
}

void MlpTrainer::gradients(const float* feat, const float* target, size_t n, float* grad, float* loss)
{
    if (n == 0 || n > (1u << 24)) throw std::invalid_argument("gradients: 1..2^24 samples");
    float *df = nullptr, *dtg = nullptr;
    check(cudaMalloc(&df, n * 3 * sizeof(float)), "samples");
    check(cudaMalloc(&dtg, n * sizeof(float)), "samples");
    const uint32_t blocks = (uint32_t)((n + TT - 1) / TT);
    try {
        check(cudaMemcpy(df, feat, n * 3 * sizeof(float), cudaMemcpyHostToDevice), "samples");
        check(cudaMemcpy(dtg, target, n * sizeof(float), cudaMemcpyHostToDevice), "samples");
        ensure_partials(blocks);
        grad_launch(df, dtg, (uint32_t)n, (uint32_t)n, true, 0, 0, blocks);
        AdamArgs a;
        std::memset(&a, 0, sizeof a);
        a.inv_batch = 1.0f / (float)n;
        a.apply = 0;
        adam_kernel<<<(MLP_NPARAM + 1 + 127) / 128, 128, 0, stream_>>>(d_params_, d_m_, d_v_, d_partials_, blocks, a,
                                                                      d_loss_);
        check(cudaGetLastError(), "adam_kernel");
        std::vector<float> g(MLP_NPARAM + 1);
        check(cudaMemcpyAsync(g.data(), d_loss_, g.size() * sizeof(float), cudaMemcpyDeviceToHost, stream_), "grad");
        check(cudaStreamSynchronize(stream_), "gradients");
        std::memcpy(grad, g.data(), MLP_NPARAM * sizeof(float));
        if (loss) *loss = g[MLP_NPARAM];
    } catch (...) {
        cudaFree(df);
        cudaFree(dtg);
        throw;
    }
    cudaFree(df);
    cudaFree(dtg);
}

const MlpDev* MlpTrainer::device_weights()
{
    if (dev_stale_) {
        MlpDev d = make_dev(params_.data(), norm);
        check(cudaMemcpy(d_dev_, &d, sizeof d, cudaMemcpyHostToDevice), "weights");
        dev_stale_ = false;
    }
    return reinterpret_cast<const MlpDev*>(d_dev_);
}

void MlpTrainer::predict(const float* feat, size_t n, float* y)
{
    if (n == 0) return;
    const MlpDev* w = device_weights();
    float *df = nullptr, *dy = nullptr;
    check(cudaMalloc(&df, n * 3 * sizeof(float)), "features");
    check(cudaMalloc(&dy, n * sizeof(float)), "outputs");
    cudaError_t e = cudaMemcpy(df, feat, n * 3 * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        predict_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream_>>>(w, df, (uint32_t)n, dy);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
    if (e == cudaSuccess) e = cudaMemcpy(y, dy, n * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(df);
    cudaFree(dy);
    check(e, "predict");
}

std::vector<uint8_t> MlpTrainer::file_bytes() const
{
    MlpFileHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, "GLMLP001", 8);
    h.nparam = MLP_NPARAM;
    h.hidden = MLP_H;
    h.norm = norm;
    std::vector<float> p(params_);
    for (int q = 0; q < MLP_NPARAM; q++)
        if (is_weight(q)) p[q] = bf16_round_host(p[q]);
    std::vector<uint8_t> out(sizeof h + MLP_NPARAM * sizeof(float));
    std::memcpy(out.data(), &h, sizeof h);
    std::memcpy(out.data() + sizeof h, p.data(), MLP_NPARAM * sizeof(float));
    return out;
}

int drift_states(const glisser_particles* pa, size_t n, double dt, double mu, int starter, const void* mlp,
                 uint32_t* evals, uint16_t* flags, cudaStream_t stream)
{
    if (!pa || n > 0xFFFFFFF0ull || !(dt > 0) || !(mu > 0)) return GLISSER_E_INVALID;
    if (starter < GLISSER_STARTER_CLASSIC || starter > GLISSER_STARTER_LEARNED) return GLISSER_E_INVALID;
    if (starter == GLISSER_STARTER_LEARNED && !mlp) return GLISSER_E_INVALID;
    if (n == 0) return GLISSER_OK;
    const unsigned grid = (unsigned)((n + 127) / 128);
    if (starter == GLISSER_STARTER_LEARNED)
        drift_states_kernel<true><<<grid, 128, 0, stream>>>(*pa, (uint32_t)n, dt, mu, starter,
                                                            reinterpret_cast<const MlpDev*>(mlp), evals, flags);
    else
        drift_states_kernel<false><<<grid, 128, 0, stream>>>(*pa, (uint32_t)n, dt, mu, starter, nullptr, evals, flags);
    return cudaGetLastError() == cudaSuccess ? GLISSER_OK : GLISSER_E_CUDA;
}

}  // namespace glisser
