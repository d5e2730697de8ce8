// Learned Kepler starter: sample logging, GPU training and device residency
// of the weights (host interface of mlp_train.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <random>
#include <string>
#include <vector>

#include "../../include/glisser.h"

namespace glisser {

struct MlpDev;

// Weights file: header followed by MLP_NPARAM floats in the flattened layout
// of mlp.cuh (the weight entries hold BF16 values; biases are FP32).
struct MlpFileHeader {
    char magic[8];             // "GLMLP001"
    uint32_t nparam;           // MLP_NPARAM
    uint32_t hidden;           // MLP_H
    glisser_mlp_norm norm;
};

// One Kepler drift per state [0, n) with the time-block kernel's drift
// routine (GLISSER_STARTER_*; `mlp` = device weights for the learned one);
// per-state evaluation counts and flags (optional device arrays).
int drift_states(const glisser_particles* pa, size_t n, double dt, double mu, int starter, const void* mlp,
                 uint32_t* evals, uint16_t* flags, cudaStream_t stream);

// Device copy of a weights file (validated), and its release.
void* mlp_upload(const std::vector<uint8_t>& file);
void mlp_free(void* dev);

class MlpTrainer {
public:
    MlpTrainer(size_t capacity, uint64_t seed);
    ~MlpTrainer();
    MlpTrainer(const MlpTrainer&) = delete;
    MlpTrainer& operator=(const MlpTrainer&) = delete;

    // Appends one sample per state: the features of the drift by dt from
    // (r, v) and the universal anomaly the plain method (classic starter,
    // FP64 Newton to the drift tolerance) converges to.  Returns the number
    // appended (limited by the remaining capacity; with a floor set, only the
    // drifts with tau^2 >= the floor are kept).
    size_t log_states(const glisser_particles& pa, size_t n, double dt, double mu, cudaStream_t stream);
    // Logs only drifts with tau^2 = dt^2 mu / r0^3 >= tau2_min (0: all): the
    // drifts where the kernels run the network.
    void set_log_floor(double tau2_min) { log_tau2_min_ = tau2_min; }
    void add_samples(const float* feat, const float* target, size_t n);
    void get_samples(float* feat, float* target, size_t first, size_t n) const;
    size_t samples() const { return n_; }
    unsigned long long plain_evals();           // Stumpff evaluations spent by the logged solves

    // Feature normalisation, output scaling and the training box from the
    // logged samples.
    void fit_norm();
    glisser_mlp_norm norm;
    bool norm_set = false;

    void get_params(float* out) const;
    void set_params(const float* in);

    // Adam on the mean squared error of the normalised output, `steps`
    // minibatches of `batch` samples drawn with replacement (seeded), learning
    // rate cosine-decayed from lr to lr_min.  losses[steps] (optional)
    // receives each step's minibatch loss.
    void train(int steps, int batch, float lr, float lr_min, uint64_t seed, float* losses);
    // Gradient of the mean loss over the given samples (device kernels).
    void gradients(const float* feat, const float* target, size_t n, float* grad, float* loss);
    // Network output y = log(s r0 / dt) by the drift's inference routine
    // (NaN outside the training box).
    void predict(const float* feat, size_t n, float* y);

    std::vector<uint8_t> file_bytes() const;
    const MlpDev* device_weights();             // current weights as the drift reads them

private:
    size_t cap_, n_ = 0;
    float *d_feat_ = nullptr, *d_target_ = nullptr;
    float *d_params_ = nullptr, *d_m_ = nullptr, *d_v_ = nullptr, *d_partials_ = nullptr, *d_loss_ = nullptr;
    unsigned long long* d_evals_ = nullptr;
    void* d_dev_ = nullptr;
    size_t partials_cap_ = 0;
    std::vector<float> params_;
    bool dev_stale_ = true;
    int adam_t_ = 0;
    double log_tau2_min_ = 0;
    cudaStream_t stream_ = nullptr;

    void ensure_partials(size_t blocks);
    void grad_launch(const float* feat, const float* target, uint32_t n, uint32_t batch, bool sequential,
                     uint64_t seed, uint32_t step, uint32_t blocks);
};

}  // namespace glisser
