// Block-loop executor: the GB300 replacement of sr::exec::Executor and
// ExecutorFacade (src/executor.cu, src/executor_facade.{h,cu}).
#pragma once
#include <cuda_runtime.h>

#include <fstream>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/glisser.h"
#include "config.h"
#include "planets.h"
#include "state_io.h"
#include "swift.h"

namespace glisser {

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Per-block timings in ms, the columns of timing.out (src/executor.cu:715-735).
struct BlockTiming {
    double enc = 0, wswift = 0, iswift = 0, swift = 0, rswift = 0, dswift = 0, io = 0, planet = 0, planetu = 0,
           encup = 0, sort = 0, dl = 0, enc2 = 0, resync = 0, cpu = 0, gpu = 0, total = 0;
};

struct FlaggedEntry {
    uint32_t id;
    uint16_t flags;
    uint32_t deathtime_index;
};

class Executor {
public:
    explicit Executor(const Config& cfg);
    ~Executor();
    Executor(const Executor&) = delete;
    Executor& operator=(const Executor&) = delete;

    Config cfg;
    std::string warnings;

    void load();                                        // load_data
    void set_planets(size_t n, const double* m, const double* r, const double* v, const uint32_t* id);
    void set_particles(size_t n, const double* r, const double* v, const uint32_t* id, const uint16_t* flags,
                       const double* deathtime);
    void init();                                        // Executor::init
    bool step_block(double* cpu_ms, double* gpu_ms);    // Executor::loop
    void finish();                                      // Executor::finish

    // host views (downloaded on demand)
    const Particles& particles();
    const Planets& planets_snapshot() const { return snapshot_; }
    const Planets& planets_live() const { return pl_; }
    const std::vector<FlaggedEntry>& last_flagged() const { return flagged_; }
    // the planet block the next step_block integrates with
    void planet_block(std::vector<double>& log, std::vector<double>& m, std::vector<uint32_t>& id,
                      std::vector<double>& rh, uint32_t& npl, uint32_t& len) const;

    double t = 0, e0 = 0;
    size_t n_alive_host() const { return n_dev_ + n_encounter_; }
    size_t n_encounter() const { return n_encounter_; }
    size_t n_total() const { return pa_.n; }
    bool initialized() const { return initialized_; }

    // Kepler starter selection (GLISSER_STARTER_*) and learned weights blob
    void set_starter(int starter, const std::vector<uint8_t>* mlp_blob);
    // Planetary history evaluated per step on the device (default) or on the
    // host (the reference's arrangement); set before init.
    void set_device_interp(bool on) { device_interp_ = on; }
    // Kepler residual tolerance |f| < tol * dt of the drift (0: 1e-13).
    void set_kepler_tolerance(double tol) { kepler_tol_ = tol; }
    // Arithmetic of the planet kick and its radius tests (GLISSER_KICK_*).
    void set_kick(int kick) { kick_ = kick; }
    int kick() const { return kick_; }
    // Track snapshots built on the device (default) or by the host writer.
    void set_device_output(bool on) { device_output_ = on; }
    // Writes a track snapshot with the particle records built on the device
    // (ms: kernels + download); false when that path does not apply (not
    // initialised, no device particles, sparse ids, or switched off).
    bool write_track_device(std::ostream& out, double* ms = nullptr);
    unsigned long long kepler_evals() const { return evals_total_; }
    // threshold-borderline radius tests (glisser_handoff.borderline) since init
    unsigned long long borderline_tests() const { return borderline_total_; }
    // drifts started from the learned starter's network guess since init
    unsigned long long learned_drifts() const { return learned_total_; }
    unsigned long long wide_drifts() const { return wide_total_; }
    unsigned long long network_blocks() const { return net_blocks_; }
    unsigned long long particle_steps() const { return psteps_total_; }
    unsigned long long launches() const { return launches_total_; }
    void* stream() const;
    // Device state the next block integrates: particles [0, n) (unflagged),
    // the step and the central mass.
    void device_view(glisser_particles* pa, size_t* n, double* dt, double* mu) const;

    std::ostream* log = nullptr;             // progress / warnings (stdout tee)
    std::ostream* encounter_out = nullptr;   // encounter.out
    std::ostream* timing_out = nullptr;      // timing.out: header at init, one row per block
    const BlockTiming& last_timing() const { return timing_; }
    // SWIFT's status arrays of the particles handed to it (Resolve-Encounters)
    const SwiftStats* swift_stats() const { return swift_ ? &swift_->stats : nullptr; }

private:
    Planets pl_;            // live planets (one block ahead of the particles after init)
    Planets snapshot_;      // planets at the particles' time
    Particles pa_;          // host mirror in device order
    std::unordered_map<uint32_t, double> deathtime_;
    std::vector<double> dt_dense_;          // deathtimes by id when ids are dense (after init)
    bool dt_dense_on_ = false;
    void set_deathtime(uint32_t id, double t);
    double get_deathtime(uint32_t id) const;
    bool loaded_pl_ = false, loaded_pa_ = false, initialized_ = false, host_dirty_ = false;

    PlanetIntegrator integ_;
    HistoryInterpolator interp_;
    std::vector<double> rh_;
    double cur_dt_ = 0, prev_dt_ = 0;
    size_t cur_tbsize_ = 0, prev_tbsize_ = 0;
    bool starting_interval_ = false;
    int starter_ = GLISSER_STARTER_SERIES;
    bool device_interp_ = true;
    double kepler_tol_ = 0;
    int kick_ = GLISSER_KICK_FLOAT_FLOAT;
    bool device_output_ = true;
    uint32_t max_id_ = 0;
    unsigned long long evals_total_ = 0, borderline_total_ = 0, learned_total_ = 0, wide_total_ = 0;
    // the learned starter's per-block dispatch: the network kernel runs when
    // the previous block had a drift outside the series starter's domain
    // (and on the first block)
    bool net_next_ = true;
    unsigned long long net_blocks_ = 0;
    unsigned long long psteps_total_ = 0;
    unsigned long long launches_total_ = 0;

    size_t n_dev_ = 0, n_encounter_ = 0;
    std::vector<FlaggedEntry> flagged_;
    BlockTiming timing_;

    // Resolve-Encounters: the SWIFT runner and the encounter particles in
    // transit (structure of arrays, as the device holds them)
    std::unique_ptr<SwiftRunner> swift_;
    struct EncounterSet {
        std::vector<double> rx, ry, rz, vx, vy, vz, ax, ay, az;
        std::vector<uint32_t> id, dti;
        std::vector<uint16_t> flags;
        void resize(size_t n);
    } enc_;
    void handle_encounters(bool from_resync, BlockTiming& tm);
    void fetch_encounters(int buf, size_t begin, size_t n);
    void store_encounters(int buf, size_t begin, size_t n);
    void encounter_accelerations(size_t n);
    void write_timing_row(const BlockTiming& tm, size_t n_enc);
    void write_timing_header();
    // encounter-flagged particles of the initial state (reported after the
    // first block, as the reference's resync reports them)
    std::vector<FlaggedEntry> initial_flagged_;

    struct Impl;
    std::unique_ptr<Impl> d_;

    void update_planets();
    void initial_accelerations(std::vector<Vec3>& acc);
    void upload_particles(const std::vector<Vec3>& acc);
    void download_particles();
};

// targets/main.cpp as a library call: runs to Final-Time writing the standard
// output folder.  Returns 0, or -1 after writing the end state on an error.
int run_main(Executor& ex, bool quiet, bool force, std::string& error);

}  // namespace glisser
