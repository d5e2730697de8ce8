// Ensemble runner: many independent planetary systems in one persistent
// launch per time block (see ensemble.cu).
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

#include "config.h"
#include "planets.h"
#include "timeblock.cuh"

namespace glisser {

class Ensemble {
public:
    Ensemble(const Config& cfg, size_t n_systems);
    ~Ensemble();
    Ensemble(const Ensemble&) = delete;
    Ensemble& operator=(const Ensemble&) = delete;

    Config cfg;
    double t = 0;

    // planets [npl] including the Sun, particles [n]; vectors are [.][3]
    void set_system(size_t s, size_t npl, const double* m, const double* r, const double* v, size_t n,
                    const double* pr, const double* pv);
    void set_shape(int cta, int ppt, uint32_t grid);
    BatchShape shape() const { return shape_; }
    void set_time_block(uint32_t len) { len_ = len; }
    uint32_t time_block() const { return len_; }
    void set_graph(bool on) { use_graph_ = on; }
    // Planet WH on the device (one warp per system; default) or on the host
    // thread pool; set before init.
    void set_device_planets(bool on);
    // Kepler residual tolerance |f| < tol * dt of the drift (0: 1e-13).
    void set_kepler_tolerance(double tol) { kepler_tol_ = tol; }
    // Arithmetic of the planet kick and its radius tests (GLISSER_KICK_*).
    void set_kick(int kick) { kick_ = kick; }
    // current planet state of system s (heliocentric)
    void planets(size_t s, std::vector<double>& m, std::vector<Vec3>& r, std::vector<Vec3>& v);
    // GLISSER_STARTER_*; the learned starter takes a weights file image
    void set_starter(int s, const std::vector<uint8_t>* mlp_file);
    void init();
    double step(double* gpu_ms);    // one block for every system

    size_t systems() const { return sys_.size(); }
    size_t alive(size_t s) const;
    size_t count(size_t s) const;
    void particles(size_t s, std::vector<Vec3>& r, std::vector<Vec3>& v, std::vector<uint32_t>& id,
                   std::vector<uint16_t>& flags);
    // The positions and velocities of every particle of every system, in
    // system order ([n][3], heliocentric; n = the ensemble's particle count),
    // through pinned staging on the ensemble's stream: put_state replaces the
    // device state the next block integrates (accelerations, flags and death
    // records are kept), take_state reads it back after the last block.
    void put_state(size_t n, const double* r, const double* v);
    void take_state(size_t cap, double* r, double* v, uint16_t* flags);
    void* stream() const;
    size_t particles_total() const { return n_; }
    // When each particle of system s was flagged: the time of the end of that
    // block as a float (the executor's deathtime stamp) and the step index
    // within it (deathtime_index); 0 for particles never flagged.
    void deaths(size_t s, std::vector<double>& deathtime, std::vector<uint32_t>& dti) const;
    unsigned long long particle_steps() const { return psteps_; }
    unsigned long long kepler_evals() const { return evals_; }
    unsigned long long borderline_tests() const { return borderline_; }
    unsigned long long learned_drifts() const { return learned_; }
    unsigned long long wide_drifts() const { return wide_; }
    unsigned long long network_blocks() const { return net_blocks_; }
    unsigned long long launches() const { return launches_; }

private:
    struct System {
        Planets pl;
        Planets snap;               // planets at the particles' time (host planet mode)
        PlanetIntegrator integ;
        std::vector<double> rh;
        std::vector<Vec3> r, v;     // start state (host)
        size_t start = 0, n = 0;
        bool set = false;
    };
    std::vector<System> sys_;
    struct Dev;
    std::unique_ptr<Dev> dev_;
    BatchShape shape_{};
    uint32_t npl_ = 0, len_ = 0, tile_ = 0;
    size_t n_ = 0, log_stride_ = 0;
    int par_ = 0;
    int starter_ = GLISSER_STARTER_SERIES;
    double kepler_tol_ = 0;
    int kick_ = GLISSER_KICK_FLOAT_FLOAT;
    bool initialized_ = false, use_graph_ = true, host_dirty_ = false, device_planets_ = true;
    std::vector<uint16_t> flags_;
    std::vector<double> deathtime_;
    std::vector<uint32_t> dti_;
    std::vector<uint32_t> killed_at_start_;   // encounter at start: deathtime stamped after the first block
    std::vector<uint32_t> ids_;
    std::vector<uint32_t> tile_first_, tile_sys_, tile_alive_;
    std::vector<uint64_t> alive_;
    unsigned long long psteps_ = 0, evals_ = 0, launches_ = 0, borderline_ = 0, learned_ = 0, wide_ = 0;
    // the learned starter's per-block dispatch (as the executor's)
    bool net_next_ = true;
    unsigned long long net_blocks_ = 0;

    void planet_block(size_t s, int par);
    void ensure_state_staging();
    void planets_all(int par);
    void planets_device(int par);
    void check_planet_status();
    void rebuild_tiles(uint32_t tile);
    uint32_t write_items(int par);
    void enqueue(int par, int starter);
};

}  // namespace glisser
