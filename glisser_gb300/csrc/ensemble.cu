// Ensemble runner: many independent planetary systems, each with its own
// planets and particles, integrated block by block in one persistent launch.
//
// Per block:
//   device, planet stream: the next block's planet WH for every system (one
//           warp per system, planets_dev.cu) writing the planet logs and
//           encounter radii the next block stages, launched just before this
//           block's kernel so its few CTAs take SMs first;
//   host  : the (system, tile) work items of the tiles that still hold alive
//           particles;
//   device: one CUDA graph per staging parity, captured once: upload of the
//           items, reset of the queue and counters, the persistent batched
//           kernel, counters back to the host (the graph waits for this
//           block's planet logs);
//   host  : the hand-off list updates the per-tile alive counts.
// Dead particles stay in place (skipped inside their tile); tiles with no
// alive particle leave the queue, so no per-system partition is needed.
// With the host planet path (more than 32 bodies, or switched off) a thread
// pool integrates every system's planets for the next block into pinned
// staging while the kernel runs, and the graph uploads them.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "config.h"
#include "ensemble.h"
#include "parallel.h"
#include "executor.h"
#include "mlp_train.h"
#include "planets_dev.h"
#include "timeblock.cuh"

namespace glisser {

namespace {

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
T* dmalloc(size_t n, const char* what)
{
    void* p = nullptr;
    ck(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), what);
    return static_cast<T*>(p);
}

template <typename T>
T* hmalloc(size_t n, const char* what)
{
    void* p = nullptr;
    ck(cudaMallocHost(&p, std::max<size_t>(n, 1) * sizeof(T)), what);
    return static_cast<T*>(p);
}

}  // namespace

struct Ensemble::Dev {
    cudaStream_t stream = nullptr;
    cudaEvent_t k0 = nullptr, k1 = nullptr;
    glisser_particles pa{};
    void* pa_base = nullptr;
    // per parity: planet blocks and items (device + pinned)
    double* d_log[2] = {};
    double* d_m[2] = {};
    double* d_rh[2] = {};
    uint32_t* d_id[2] = {};
    BatchItem* d_items[2] = {};
    uint32_t* d_nitems[2] = {};
    double* h_log[2] = {};
    double* h_m[2] = {};
    double* h_rh[2] = {};
    uint32_t* h_id[2] = {};
    BatchItem* h_items[2] = {};
    uint32_t* h_nitems[2] = {};
    uint32_t* d_ctr = nullptr;      // [0] hand-off count, [1] status, [2] queue
    unsigned long long* d_evals = nullptr;
    uint32_t* h_ctr = nullptr;
    unsigned long long* h_evals = nullptr;
    uint32_t *d_ho_index = nullptr, *d_ho_id = nullptr, *d_ho_dti = nullptr;
    uint16_t* d_ho_flags = nullptr;
    uint32_t *h_ho_index = nullptr, *h_ho_dti = nullptr;
    uint16_t* h_ho_flags = nullptr;
    // one graph per staging parity and starter kernel (slot = parity + 2 x
    // network kernel)
    cudaGraphExec_t graph[4] = {};
    BatchShape graph_shape[4] = {};
    uint32_t graph_len[4] = {};
    int graph_starter[4] = { -1, -1, -1, -1 };
    double graph_tol[4] = { -1, -1, -1, -1 };
    int graph_kick[4] = { -1, -1, -1, -1 };
    void* d_mlp = nullptr;            // learned-starter weights
    // device planet integrator state ([S][npl] arrays, one allocation)
    PlanetSysDev pl{};
    double* snap[6] = {};             // r, v at the particles' time
    void* pl_base = nullptr;
    uint32_t* h_status = nullptr;
    cudaStream_t pstream = nullptr;
    cudaEvent_t planets_done = nullptr;
    int mlp_version = 0, graph_mlp[4] = { 0, 0, 0, 0 };
    double* h_state = nullptr;        // pinned staging of whole-ensemble state transfers
    uint16_t* h_state_flags = nullptr;

    ~Dev()
    {
        cudaFreeHost(h_state);
        cudaFreeHost(h_state_flags);
        mlp_free(d_mlp);
        cudaFree(pl_base);
        cudaFreeHost(h_status);
        if (planets_done) cudaEventDestroy(planets_done);
        if (pstream) cudaStreamDestroy(pstream);
        for (int g = 0; g < 4; g++)
            if (graph[g]) cudaGraphExecDestroy(graph[g]);
        for (int b = 0; b < 2; b++) {
            cudaFree(d_log[b]); cudaFree(d_m[b]); cudaFree(d_rh[b]); cudaFree(d_id[b]);
            cudaFree(d_items[b]); cudaFree(d_nitems[b]);
            cudaFreeHost(h_log[b]); cudaFreeHost(h_m[b]); cudaFreeHost(h_rh[b]); cudaFreeHost(h_id[b]);
            cudaFreeHost(h_items[b]); cudaFreeHost(h_nitems[b]);
        }
        cudaFree(pa_base);
        cudaFree(d_ctr); cudaFree(d_evals); cudaFree(d_ho_index); cudaFree(d_ho_id); cudaFree(d_ho_dti);
        cudaFree(d_ho_flags);
        cudaFreeHost(h_ctr); cudaFreeHost(h_evals); cudaFreeHost(h_ho_index); cudaFreeHost(h_ho_dti);
        cudaFreeHost(h_ho_flags);
        if (k0) cudaEventDestroy(k0);
        if (k1) cudaEventDestroy(k1);
        if (stream) cudaStreamDestroy(stream);
    }
};

Ensemble::Ensemble(const Config& c, size_t n_systems) : cfg(c), sys_(n_systems), dev_(new Dev())
{
    if (n_systems == 0) throw std::invalid_argument("an ensemble needs at least one system");
    shape_ = BatchShape{ 128, 1, 0 };
}

Ensemble::~Ensemble() = default;

void Ensemble::set_device_planets(bool on)
{
    if (initialized_) throw std::invalid_argument("set_device_planets: call before init");
    device_planets_ = on;
}

void Ensemble::planets(size_t s, std::vector<double>& m, std::vector<Vec3>& r, std::vector<Vec3>& v)
{
    if (s >= sys_.size()) throw std::invalid_argument("system index out of range");
    const System& y = sys_[s];
    if (!initialized_ || !device_planets_) {
        const Planets& src_pl = initialized_ ? y.snap : y.pl;
        m = src_pl.m;
        r = src_pl.r;
        v = src_pl.v;
        return;
    }
    m = y.pl.m;                     // masses do not change
    r.assign(npl_, Vec3{ 0, 0, 0 });
    v.assign(npl_, Vec3{ 0, 0, 0 });
    // the device holds the planets one block ahead of the particles: the
    // state at the particles' time is the start of the staged block
    Dev& d = *dev_;
    ck(cudaStreamSynchronize(d.stream), "sync");
    ck(cudaStreamSynchronize(d.pstream), "sync");
    const size_t at = s * npl_;
    std::vector<double> c(6 * npl_);
    double* const* src = d.snap;
    for (int k = 0; k < 6; k++)
        ck(cudaMemcpy(c.data() + k * npl_, src[k] + at, npl_ * sizeof(double), cudaMemcpyDeviceToHost), "planets");
    for (uint32_t j = 0; j < npl_; j++) {
        r[j] = Vec3{ c[j], c[npl_ + j], c[2 * npl_ + j] };
        v[j] = Vec3{ c[3 * npl_ + j], c[4 * npl_ + j], c[5 * npl_ + j] };
    }
}

void Ensemble::set_starter(int s, const std::vector<uint8_t>* mlp_file)
{
    if (s < GLISSER_STARTER_CLASSIC || s > GLISSER_STARTER_LEARNED) throw std::invalid_argument("unknown starter");
    if (s == GLISSER_STARTER_LEARNED) {
        if (!mlp_file) throw std::invalid_argument("the learned starter needs a weights file");
        void* w = mlp_upload(*mlp_file);
        mlp_free(dev_->d_mlp);
        dev_->d_mlp = w;
        dev_->mlp_version++;
    }
    starter_ = s;
    net_next_ = true;
}

void Ensemble::set_system(size_t s, size_t npl, const double* m, const double* r, const double* v, size_t n,
                          const double* pr, const double* pv)
{
    if (initialized_) throw std::runtime_error("systems can only be set before init");
    if (s >= sys_.size()) throw std::invalid_argument("system index out of range");
    System& y = sys_[s];
    y.pl.resize(npl);
    y.pl.n_alive = npl;
    for (size_t i = 0; i < npl; i++) {
        y.pl.m[i] = m[i] * cfg.big_g;
        y.pl.r[i] = Vec3{ r[3 * i], r[3 * i + 1], r[3 * i + 2] };
        y.pl.v[i] = Vec3{ v[3 * i], v[3 * i + 1], v[3 * i + 2] };
        y.pl.id[i] = (uint32_t)i;
    }
    y.r.resize(n);
    y.v.resize(n);
    for (size_t k = 0; k < n; k++) {
        y.r[k] = Vec3{ pr[3 * k], pr[3 * k + 1], pr[3 * k + 2] };
        y.v[k] = Vec3{ pv[3 * k], pv[3 * k + 1], pv[3 * k + 2] };
    }
    y.set = true;
}

void Ensemble::set_shape(int cta, int ppt, uint32_t grid)
{
    if (!(cta == 64 || cta == 128 || cta == 256) || !(ppt == 1 || ppt == 2))
        throw std::invalid_argument("shape: cta must be 64, 128 or 256 and ppt 1 or 2");
    if (initialized_ && (uint32_t)(cta * ppt) != tile_) rebuild_tiles(cta * ppt);
    shape_ = BatchShape{ cta, ppt, grid };
}

// Planet block of one system for the next cur_len steps (host, one thread).
void Ensemble::planet_block(size_t s, int par)
{
    Dev& d = *dev_;
    System& y = sys_[s];
    const uint32_t npl = npl_;
    y.snap = y.pl;
    y.integ.encounter_radii(y.pl, cfg.cull_radius, cfg.encounter_sphere_factor, y.rh);
    double* log = d.h_log[par] + s * log_stride_;
    for (uint32_t k = 0; k < len_; k++) {
        Vec3 h0 = y.integ.step(y.pl, cfg.dt);
        double* rec = log + (size_t)k * 3 * npl;
        rec[0] = h0.x; rec[1] = h0.y; rec[2] = h0.z;
        for (uint32_t j = 1; j < npl; j++) {
            rec[3 * j] = y.pl.r[j].x;
            rec[3 * j + 1] = y.pl.r[j].y;
            rec[3 * j + 2] = y.pl.r[j].z;
        }
    }
    for (uint32_t j = 0; j < npl; j++) {
        d.h_m[par][s * npl + j] = y.pl.m[j];
        d.h_rh[par][s * npl + j] = y.rh[j];
        d.h_id[par][s * npl + j] = y.pl.id[j];
    }
}

void Ensemble::planets_all(int par)
{
    const size_t S = sys_.size();
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    size_t nth = std::min<size_t>(hw, S);
    std::atomic<size_t> next{ 0 };
    std::vector<std::exception_ptr> errs(nth);
    auto work = [&](size_t w) {
        try {
            for (size_t s = next++; s < S; s = next++) planet_block(s, par);
        } catch (...) {
            errs[w] = std::current_exception();
        }
    };
    std::vector<std::thread> th;
    for (size_t w = 1; w < nth; w++) th.emplace_back(work, w);
    work(0);
    for (auto& t : th) t.join();
    for (auto& e : errs)
        if (e) std::rethrow_exception(e);
}

// The next block's planet logs and encounter radii on the device (one warp
// per system), on the planet stream; the block's kernel waits for it.
void Ensemble::planets_device(int par)
{
    Dev& d = *dev_;
    const size_t S = sys_.size(), cnt = S * npl_;
    const double* src[6] = { d.pl.rx, d.pl.ry, d.pl.rz, d.pl.vx, d.pl.vy, d.pl.vz };
    for (int k = 0; k < 6; k++)
        ck(cudaMemcpyAsync(d.snap[k], src[k], cnt * sizeof(double), cudaMemcpyDeviceToDevice, d.pstream), "snapshot");
    ck(launch_planet_wh(d.pl, (uint32_t)S, npl_, len_, cfg.dt, cfg.cull_radius, cfg.encounter_sphere_factor,
                        d.d_log[par], log_stride_, d.d_rh[par], d.pstream),
       "planet kernel");
    launches_ += 1;
    ck(cudaMemcpyAsync(d.h_status, d.pl.status, S * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.pstream), "status");
    ck(cudaEventRecord(d.planets_done, d.pstream), "event");
}

void Ensemble::check_planet_status()
{
    Dev& d = *dev_;
    ck(cudaEventSynchronize(d.planets_done), "planet kernel");
    for (size_t s = 0; s < sys_.size(); s++) {
        uint32_t st = d.h_status[s];
        if (!st) continue;
        uint32_t planet = st >> 8;
        if ((st & 0xFF) == 1) throw StateError("unbound orbit of planet " + std::to_string(planet) + " (system " +
                                               std::to_string(s) + ")");
        throw StateError("Unconverging kepler (system " + std::to_string(s) + ", planet " + std::to_string(planet) +
                         ")");
    }
}

void Ensemble::rebuild_tiles(uint32_t tile)
{
    tile_ = tile;
    tile_alive_.clear();
    tile_first_.clear();
    tile_sys_.clear();
    for (size_t s = 0; s < sys_.size(); s++) {
        const System& y = sys_[s];
        for (size_t f = 0; f < y.n; f += tile) {
            uint32_t cnt = (uint32_t)std::min<size_t>(tile, y.n - f);
            uint32_t alive = 0;
            for (uint32_t q = 0; q < cnt; q++) alive += flags_[y.start + f + q] == 0;
            tile_first_.push_back((uint32_t)(y.start + f));
            tile_sys_.push_back((uint32_t)s);
            tile_alive_.push_back(alive);
            (void)cnt;
        }
    }
}

uint32_t Ensemble::write_items(int par)
{
    Dev& d = *dev_;
    uint32_t k = 0;
    for (size_t t = 0; t < tile_first_.size(); t++) {
        if (tile_alive_[t] == 0) continue;
        const System& y = sys_[tile_sys_[t]];
        uint32_t end = (uint32_t)(y.start + y.n);
        d.h_items[par][k++] = BatchItem{ tile_sys_[t], tile_first_[t], std::min(tile_, end - tile_first_[t]), 0 };
    }
    *d.h_nitems[par] = k;
    return k;
}

void Ensemble::init()
{
    if (initialized_) throw std::runtime_error("init called twice");
    for (auto& y : sys_)
        if (!y.set) throw std::runtime_error("every system must be set before init");
    npl_ = (uint32_t)sys_[0].pl.n;
    for (auto& y : sys_)
        if (y.pl.n != npl_) throw std::runtime_error("all systems of an ensemble need the same planet count");
    if (npl_ < 1 || npl_ > (uint32_t)MAX_PLANETS) throw StateError("planet count out of range");
    len_ = cfg.tbsize;
    if (len_ == 0) throw std::runtime_error("Time-Block-Size must be positive");
    Dev& d = *dev_;

    // heliocentric states, planet integrators, start accelerations (the
    // reference's WHIntegrator ctor, src/wh.cpp:498-577)
    size_t total = 0;
    for (auto& y : sys_) {
        y.start = total;
        y.n = y.r.size();
        total += y.n;
    }
    n_ = total;
    std::vector<double> col(9 * std::max<size_t>(total, 1));
    flags_.assign(total, 0);
    deathtime_.assign(total, 0.0);
    dti_.assign(total, 0u);
    ids_.resize(total);
    for (size_t s = 0; s < sys_.size(); s++) {
        System& y = sys_[s];
        Vec3 r0 = y.pl.r[0], v0 = y.pl.v[0];
        for (size_t i = 0; i < y.pl.n; i++) {
            y.pl.r[i] -= r0;
            y.pl.v[i] -= v0;
        }
        y.integ.init(y.pl);
        y.integ.encounter_radii(y.pl, cfg.cull_radius, cfg.encounter_sphere_factor, y.rh);
        Vec3 h0 = y.integ.accelerations(y.pl);
        for (size_t k = 0; k < y.n; k++) {
            size_t g = y.start + k;
            Vec3 r = y.r[k] - r0, v = y.v[k] - v0;
            Vec3 a = h0;
            uint16_t fl = 0;
            for (size_t j = 1; j < y.pl.n_alive; j++) {
                Vec3 dr = r - y.pl.r[j];
                double r2 = dr.lensq();
                double irij3 = 1. / (r2 * std::sqrt(r2));
                a -= dr * (y.pl.m[j] * irij3);
                if (r2 < y.rh[j] * y.rh[j]) fl = (uint16_t)((j << 8) | 0x0001);
            }
            double r2 = r.lensq();
            if (r2 < y.rh[0] * y.rh[0]) fl = 0x0001;
            if (r2 > cfg.outer_radius * cfg.outer_radius) fl = 0x0002;
            double* c = col.data();
            c[g] = r.x; c[total + g] = r.y; c[2 * total + g] = r.z;
            c[3 * total + g] = v.x; c[4 * total + g] = v.y; c[5 * total + g] = v.z;
            c[6 * total + g] = a.x; c[7 * total + g] = a.y; c[8 * total + g] = a.z;
            // a particle inside an encounter radius at start is removed at the
            // end of the first block, as the reference's KillEncounterKernel
            // does with the encounter particles its initial partition leaves in
            // the alive range (src/executor.cu:181-187, 63-78): flagged dead
            // here, its deathtime stamped when the first block ends
            if (fl & 0x01) {
                fl = (uint16_t)((fl & 0xFF00) | 0x80);
                killed_at_start_.push_back((uint32_t)g);
            }
            flags_[g] = fl;
            ids_[g] = (uint32_t)k;
        }
        alive_.push_back(0);
        for (size_t k = 0; k < y.n; k++) alive_.back() += flags_[y.start + k] == 0;
    }

    ck(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking), "stream");
    ck(cudaEventCreate(&d.k0), "event");
    ck(cudaEventCreate(&d.k1), "event");
    size_t cap = std::max<size_t>(total, 1);
    size_t bytes = cap * (9 * sizeof(double) + 2 * sizeof(uint32_t) + sizeof(uint16_t)) + 1024;
    ck(cudaMalloc(&d.pa_base, bytes), "cudaMalloc particles");
    char* q = static_cast<char*>(d.pa_base);
    double** dbl[9] = { &d.pa.rx, &d.pa.ry, &d.pa.rz, &d.pa.vx, &d.pa.vy, &d.pa.vz, &d.pa.ax, &d.pa.ay, &d.pa.az };
    for (int k = 0; k < 9; k++) {
        *dbl[k] = reinterpret_cast<double*>(q);
        q += cap * sizeof(double);
    }
    d.pa.deathtime_index = reinterpret_cast<uint32_t*>(q);
    q += cap * sizeof(uint32_t);
    d.pa.id = reinterpret_cast<uint32_t*>(q);
    q += cap * sizeof(uint32_t);
    d.pa.flags = reinterpret_cast<uint16_t*>(q);
    for (int k = 0; k < 9; k++)
        ck(cudaMemcpy(*dbl[k], col.data() + k * total, total * sizeof(double), cudaMemcpyHostToDevice), "upload");
    ck(cudaMemcpy(d.pa.flags, flags_.data(), total * sizeof(uint16_t), cudaMemcpyHostToDevice), "upload flags");
    ck(cudaMemcpy(d.pa.id, ids_.data(), total * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload ids");
    ck(cudaMemset(d.pa.deathtime_index, 0, total * sizeof(uint32_t)), "memset");

    // planet blocks: per system stride rounded to 16 bytes
    uint32_t recs = (len_ + 1u) & ~1u;
    log_stride_ = (size_t)recs * 3 * npl_;
    log_stride_ = (log_stride_ + 1) & ~(size_t)1;
    size_t S = sys_.size();
    size_t max_tiles = total / 64 + S + 1;
    for (int b = 0; b < 2; b++) {
        d.d_log[b] = dmalloc<double>(S * log_stride_, "cudaMalloc log");
        d.d_m[b] = dmalloc<double>(S * npl_, "cudaMalloc m");
        d.d_rh[b] = dmalloc<double>(S * npl_, "cudaMalloc rh");
        d.d_id[b] = dmalloc<uint32_t>(S * npl_, "cudaMalloc id");
        d.d_items[b] = dmalloc<BatchItem>(max_tiles, "cudaMalloc items");
        d.d_nitems[b] = dmalloc<uint32_t>(1, "cudaMalloc items");
        d.h_log[b] = hmalloc<double>(S * log_stride_, "pinned log");
        std::memset(d.h_log[b], 0, S * log_stride_ * sizeof(double));
        d.h_m[b] = hmalloc<double>(S * npl_, "pinned");
        d.h_rh[b] = hmalloc<double>(S * npl_, "pinned");
        d.h_id[b] = hmalloc<uint32_t>(S * npl_, "pinned");
        d.h_items[b] = hmalloc<BatchItem>(max_tiles, "pinned");
        d.h_nitems[b] = hmalloc<uint32_t>(1, "pinned");
    }
    d.d_ctr = dmalloc<uint32_t>(8, "cudaMalloc counters");
    d.d_evals = dmalloc<unsigned long long>(4, "cudaMalloc evals");
    d.h_ctr = hmalloc<uint32_t>(8, "pinned");
    d.h_evals = hmalloc<unsigned long long>(4, "pinned");
    d.d_ho_index = dmalloc<uint32_t>(cap, "cudaMalloc hand-off");
    d.d_ho_id = dmalloc<uint32_t>(cap, "cudaMalloc hand-off");
    d.d_ho_dti = dmalloc<uint32_t>(cap, "cudaMalloc hand-off");
    d.d_ho_flags = dmalloc<uint16_t>(cap, "cudaMalloc hand-off");
    d.h_ho_index = hmalloc<uint32_t>(cap, "pinned");
    d.h_ho_dti = hmalloc<uint32_t>(cap, "pinned");
    d.h_ho_flags = hmalloc<uint16_t>(cap, "pinned");
    rebuild_tiles(shape_.cta * shape_.ppt);
    if (device_planets_ && npl_ > PLANET_WH_MAX_NPL) device_planets_ = false;   // host planets beyond 32 bodies
    if (device_planets_) {
        // planet state for the device integrator, masses and ids (constant)
        const size_t cnt = S * npl_;
        ck(cudaStreamCreateWithFlags(&d.pstream, cudaStreamNonBlocking), "stream");
        ck(cudaEventCreateWithFlags(&d.planets_done, cudaEventDisableTiming), "event");
        ck(cudaMalloc(&d.pl_base, cnt * 20 * sizeof(double) + S * sizeof(uint32_t)), "cudaMalloc planets");
        double* q = static_cast<double*>(d.pl_base);
        double** arr[14] = { &d.pl.rx, &d.pl.ry, &d.pl.rz, &d.pl.vx, &d.pl.vy, &d.pl.vz, &d.pl.ax, &d.pl.ay,
                             &d.pl.az, &d.pl.jx, &d.pl.jy, &d.pl.jz, &d.pl.m, &d.pl.eta };
        for (int k = 0; k < 14; k++) {
            *arr[k] = q;
            q += cnt;
        }
        for (int k = 0; k < 6; k++) {
            d.snap[k] = q;
            q += cnt;
        }
        d.pl.status = reinterpret_cast<uint32_t*>(q);
        d.h_status = hmalloc<uint32_t>(S, "pinned");
        std::vector<double> h(14 * cnt);
        for (size_t s = 0; s < S; s++) {
            System& y = sys_[s];
            const auto& rj = y.integ.jacobi_r();
            const auto& acc = y.integ.acc();
            const auto& eta = y.integ.eta();
            for (uint32_t j = 0; j < npl_; j++) {
                const size_t at = s * npl_ + j;
                const Vec3 a = j ? acc[j] : Vec3{ 0, 0, 0 };
                const double vals[14] = { y.pl.r[j].x, y.pl.r[j].y, y.pl.r[j].z, y.pl.v[j].x, y.pl.v[j].y,
                                          y.pl.v[j].z, a.x, a.y, a.z, rj[j].x, rj[j].y, rj[j].z, y.pl.m[j], eta[j] };
                for (int k = 0; k < 14; k++) h[k * cnt + at] = vals[k];
                for (int b = 0; b < 2; b++) {
                    d.h_m[b][at] = y.pl.m[j];
                    d.h_id[b][at] = y.pl.id[j];
                }
            }
        }
        ck(cudaMemcpy(d.pl.rx, h.data(), 14 * cnt * sizeof(double), cudaMemcpyHostToDevice), "upload planets");
        ck(cudaMemset(d.pl.status, 0, S * sizeof(uint32_t)), "memset");
        for (int b = 0; b < 2; b++) {
            ck(cudaMemcpy(d.d_m[b], d.h_m[b], cnt * sizeof(double), cudaMemcpyHostToDevice), "upload m");
            ck(cudaMemcpy(d.d_id[b], d.h_id[b], cnt * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload ids");
        }
    }
    initialized_ = true;
    par_ = 0;
    if (device_planets_) {
        planets_device(par_);
        check_planet_status();
    } else {
        planets_all(par_);
    }
}

// Enqueues one block on the stream: uploads, counter reset, kernel, counters
// back.  `starter` is the block's kernel: the learned one, or the series
// one in its place on a block after one without drifts outside the series
// starter's domain.
void Ensemble::enqueue(int par, int starter)
{
    Dev& d = *dev_;
    const size_t S = sys_.size();
    if (!device_planets_) {
        ck(cudaMemcpyAsync(d.d_log[par], d.h_log[par], S * log_stride_ * sizeof(double), cudaMemcpyHostToDevice,
                           d.stream), "upload log");
        ck(cudaMemcpyAsync(d.d_m[par], d.h_m[par], S * npl_ * sizeof(double), cudaMemcpyHostToDevice, d.stream), "m");
        ck(cudaMemcpyAsync(d.d_rh[par], d.h_rh[par], S * npl_ * sizeof(double), cudaMemcpyHostToDevice, d.stream),
           "rh");
        ck(cudaMemcpyAsync(d.d_id[par], d.h_id[par], S * npl_ * sizeof(uint32_t), cudaMemcpyHostToDevice, d.stream),
           "id");
    }
    size_t max_tiles = n_ / 64 + S + 1;
    ck(cudaMemcpyAsync(d.d_items[par], d.h_items[par], max_tiles * sizeof(BatchItem), cudaMemcpyHostToDevice,
                       d.stream), "items");
    ck(cudaMemcpyAsync(d.d_nitems[par], d.h_nitems[par], sizeof(uint32_t), cudaMemcpyHostToDevice, d.stream), "n");
    ck(cudaMemsetAsync(d.d_ctr, 0, 8 * sizeof(uint32_t), d.stream), "memset");
    ck(cudaMemsetAsync(d.d_evals, 0, 4 * sizeof(unsigned long long), d.stream), "memset");
    BatchSystems sy{ d.d_log[par], log_stride_, d.d_m[par], d.d_rh[par], d.d_id[par] };
    glisser_step_params sp{};
    sp.dt = cfg.dt;
    sp.outer_radius = cfg.outer_radius;
    sp.starter = starter;
    sp.kill_encounters = 1;
    sp.mlp = starter == GLISSER_STARTER_LEARNED ? d.d_mlp : nullptr;
    sp.kepler_tol = kepler_tol_;
    sp.kick = kick_;
    glisser_handoff ho{};
    ho.count = d.d_ctr;
    ho.status = d.d_ctr + 1;
    ho.index = d.d_ho_index;
    ho.id = d.d_ho_id;
    ho.flags = d.d_ho_flags;
    ho.deathtime_index = d.d_ho_dti;
    ho.capacity = (uint32_t)std::max<size_t>(n_, 1);
    ho.evals = d.d_evals;
    ho.borderline = d.d_evals + 1;
    ho.learned = d.d_evals + 2;
    ho.wide = d.d_evals + 3;
    int rc = launch_batched(&d.pa, sy, d.d_items[par], d.d_nitems[par], d.d_ctr + 2, npl_, len_, &sp, &ho, shape_,
                            d.stream);
    if (rc != GLISSER_OK) throw CudaError(std::string("batched launch failed: ") + timeblock_error());
    ck(cudaMemcpyAsync(d.h_ctr, d.d_ctr, 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.stream), "counters");
    ck(cudaMemcpyAsync(d.h_evals, d.d_evals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, d.stream),
       "evals");
}

double Ensemble::step(double* gpu_ms)
{
    if (!initialized_) throw std::runtime_error("step before init");
    Dev& d = *dev_;
    const int par = par_;
    uint32_t nitems = write_items(par);
    uint64_t before_alive = 0;
    for (auto a : alive_) before_alive += a;
    if (device_planets_) {
        // this block waits for its planet logs; the next block's planets are
        // launched before this block's kernel so that their few CTAs take SMs
        // first and run alongside the persistent kernel
        ck(cudaStreamWaitEvent(d.stream, d.planets_done, 0), "wait planets");
        planets_device(par ^ 1);
    }
    if (nitems > 0) {
        const bool net = starter_ == GLISSER_STARTER_LEARNED && net_next_;
        const int starter = starter_ == GLISSER_STARTER_LEARNED && !net ? GLISSER_STARTER_SERIES : starter_;
        net_blocks_ += net;
        ck(cudaEventRecord(d.k0, d.stream), "event");
        if (use_graph_) {
            const int slot = par + (net ? 2 : 0);
            const BatchShape& gs = d.graph_shape[slot];
            bool stale = !d.graph[slot] || gs.cta != shape_.cta || gs.ppt != shape_.ppt || gs.grid != shape_.grid ||
                         d.graph_len[slot] != len_ || d.graph_starter[slot] != starter ||
                         d.graph_mlp[slot] != d.mlp_version || d.graph_tol[slot] != kepler_tol_ ||
                         d.graph_kick[slot] != kick_;
            if (stale) {
                if (d.graph[slot]) cudaGraphExecDestroy(d.graph[slot]);
                d.graph[slot] = nullptr;
                cudaGraph_t g;
                ck(cudaStreamBeginCapture(d.stream, cudaStreamCaptureModeRelaxed), "begin capture");
                enqueue(par, starter);
                ck(cudaStreamEndCapture(d.stream, &g), "end capture");
                ck(cudaGraphInstantiate(&d.graph[slot], g, 0), "instantiate");
                cudaGraphDestroy(g);
                d.graph_len[slot] = len_;
                d.graph_shape[slot] = shape_;
                d.graph_starter[slot] = starter;
                d.graph_mlp[slot] = d.mlp_version;
                d.graph_tol[slot] = kepler_tol_;
                d.graph_kick[slot] = kick_;
            }
            ck(cudaGraphLaunch(d.graph[slot], d.stream), "graph launch");
            launches_ += 1;
        } else {
            enqueue(par, starter);
            launches_ += 1;
        }
        ck(cudaEventRecord(d.k1, d.stream), "event");
    }
    // the next block's planets while the kernel runs
    t += cfg.dt * len_;
    par_ ^= 1;
    if (!device_planets_) planets_all(par_);
    float ms = 0;
    if (device_planets_) check_planet_status();
    if (nitems > 0) {
        ck(cudaStreamSynchronize(d.stream), "block");
        ck(cudaEventElapsedTime(&ms, d.k0, d.k1), "elapsed");
        if (d.h_ctr[1]) throw CudaError("batched kernel reported a planet-log staging timeout");
        uint32_t k = std::min<uint32_t>(d.h_ctr[0], (uint32_t)std::max<size_t>(n_, 1));
        evals_ += d.h_evals[0];
        borderline_ += d.h_evals[1];
        learned_ += d.h_evals[2];
        wide_ += d.h_evals[3];
        net_next_ = d.h_evals[3] > 0;
        uint64_t dti_sum = 0;
        if (k) {
            ck(cudaMemcpy(d.h_ho_index, d.d_ho_index, k * sizeof(uint32_t), cudaMemcpyDeviceToHost), "hand-off");
            ck(cudaMemcpy(d.h_ho_dti, d.d_ho_dti, k * sizeof(uint32_t), cudaMemcpyDeviceToHost), "hand-off");
            ck(cudaMemcpy(d.h_ho_flags, d.d_ho_flags, k * sizeof(uint16_t), cudaMemcpyDeviceToHost), "hand-off");
            const float tf = (float)t;     // block end, stamped as the executor does
            for (uint32_t q = 0; q < k; q++) {
                uint32_t g = d.h_ho_index[q];
                bool was_alive = flags_[g] == 0;
                flags_[g] = d.h_ho_flags[q];
                dti_sum += d.h_ho_dti[q];
                deathtime_[g] = tf;
                dti_[g] = d.h_ho_dti[q];
                if (was_alive && flags_[g] != 0) {
                    // locate the tile and the system of particle g
                    size_t t = std::upper_bound(tile_first_.begin(), tile_first_.end(), g) - tile_first_.begin() - 1;
                    tile_alive_[t]--;
                    alive_[tile_sys_[t]]--;
                }
            }
        }
        if (!killed_at_start_.empty()) {
            const float tf = (float)t;
            for (uint32_t g : killed_at_start_) deathtime_[g] = tf;
            killed_at_start_.clear();
        }
        uint64_t after_alive = 0;
        for (auto a : alive_) after_alive += a;
        // survivors advanced the whole block, the newly flagged their index
        psteps_ += (before_alive - (before_alive - after_alive)) * (uint64_t)len_ + dti_sum;
        host_dirty_ = true;
    }
    if (gpu_ms) *gpu_ms = ms;
    return ms;
}

void Ensemble::particles(size_t s, std::vector<Vec3>& r, std::vector<Vec3>& v, std::vector<uint32_t>& id,
                         std::vector<uint16_t>& flags)
{
    if (s >= sys_.size()) throw std::invalid_argument("system index out of range");
    if (!initialized_) throw std::runtime_error("particles before init");
    Dev& d = *dev_;
    const System& y = sys_[s];
    std::vector<double> c(6 * y.n);
    double* src[6] = { d.pa.rx, d.pa.ry, d.pa.rz, d.pa.vx, d.pa.vy, d.pa.vz };
    ck(cudaStreamSynchronize(d.stream), "sync");
    for (int k = 0; k < 6; k++)
        ck(cudaMemcpy(c.data() + k * y.n, src[k] + y.start, y.n * sizeof(double), cudaMemcpyDeviceToHost), "download");
    r.resize(y.n);
    v.resize(y.n);
    id.resize(y.n);
    flags.resize(y.n);
    ck(cudaMemcpy(id.data(), d.pa.id + y.start, y.n * sizeof(uint32_t), cudaMemcpyDeviceToHost), "download ids");
    ck(cudaMemcpy(flags.data(), d.pa.flags + y.start, y.n * sizeof(uint16_t), cudaMemcpyDeviceToHost), "download");
    for (size_t k = 0; k < y.n; k++) {
        r[k] = Vec3{ c[k], c[y.n + k], c[2 * y.n + k] };
        v[k] = Vec3{ c[3 * y.n + k], c[4 * y.n + k], c[5 * y.n + k] };
    }
}

void* Ensemble::stream() const { return dev_ ? (void*)dev_->stream : nullptr; }

void Ensemble::ensure_state_staging()
{
    Dev& d = *dev_;
    if (d.h_state) return;
    d.h_state = hmalloc<double>(6 * std::max<size_t>(n_, 1), "pinned state");
    d.h_state_flags = hmalloc<uint16_t>(std::max<size_t>(n_, 1), "pinned state");
}

void Ensemble::put_state(size_t n, const double* r, const double* v)
{
    if (!initialized_) throw std::runtime_error("put_state before init");
    if (n != n_) throw std::invalid_argument("put_state: particle count differs from the ensemble's");
    ensure_state_staging();
    Dev& d = *dev_;
    double* st = d.h_state;
    // a state at tau^2 = dt^2 mu / r^3 >= 0.01 about the heaviest central
    // mass brings the learned starter's network kernel back for the next block
    double mu = 0;
    for (const System& y : sys_) mu = std::max(mu, y.pl.m.empty() ? 0.0 : y.pl.m[0]);
    const double rw = std::cbrt(100.0 * cfg.dt * cfg.dt * mu), rw2 = rw * rw;
    std::atomic<bool> near{ false };
    parallel_for(n, [&](size_t b, size_t e) {
        bool nr = false;
        for (size_t k = b; k < e; k++) {
            st[k] = r[3 * k]; st[n + k] = r[3 * k + 1]; st[2 * n + k] = r[3 * k + 2];
            st[3 * n + k] = v[3 * k]; st[4 * n + k] = v[3 * k + 1]; st[5 * n + k] = v[3 * k + 2];
            nr |= r[3 * k] * r[3 * k] + r[3 * k + 1] * r[3 * k + 1] + r[3 * k + 2] * r[3 * k + 2] <= rw2;
        }
        if (nr) near.store(true, std::memory_order_relaxed);
    });
    if (near.load()) net_next_ = true;
    double* dst[6] = { d.pa.rx, d.pa.ry, d.pa.rz, d.pa.vx, d.pa.vy, d.pa.vz };
    for (int k = 0; k < 6; k++)
        ck(cudaMemcpyAsync(dst[k], st + k * n, n * sizeof(double), cudaMemcpyHostToDevice, d.stream), "upload state");
    // the next block's kernel runs on the same stream, after the copies
}

void Ensemble::take_state(size_t cap, double* r, double* v, uint16_t* flags)
{
    if (!initialized_) throw std::runtime_error("take_state before init");
    if (cap < n_) throw std::invalid_argument("take_state: room for fewer particles than the ensemble holds");
    ensure_state_staging();
    Dev& d = *dev_;
    const size_t n = n_;
    double* st = d.h_state;
    const double* src[6] = { d.pa.rx, d.pa.ry, d.pa.rz, d.pa.vx, d.pa.vy, d.pa.vz };
    for (int k = 0; k < 6; k++)
        ck(cudaMemcpyAsync(st + k * n, src[k], n * sizeof(double), cudaMemcpyDeviceToHost, d.stream), "download state");
    if (flags)
        ck(cudaMemcpyAsync(d.h_state_flags, d.pa.flags, n * sizeof(uint16_t), cudaMemcpyDeviceToHost, d.stream),
           "download flags");
    ck(cudaStreamSynchronize(d.stream), "download sync");
    parallel_for(n, [&](size_t b, size_t e) {
        for (size_t k = b; k < e; k++) {
            if (r) { r[3 * k] = st[k]; r[3 * k + 1] = st[n + k]; r[3 * k + 2] = st[2 * n + k]; }
            if (v) { v[3 * k] = st[3 * n + k]; v[3 * k + 1] = st[4 * n + k]; v[3 * k + 2] = st[5 * n + k]; }
            if (flags) flags[k] = d.h_state_flags[k];
        }
    });
}

void Ensemble::deaths(size_t s, std::vector<double>& deathtime, std::vector<uint32_t>& dti) const
{
    if (s >= sys_.size()) throw std::invalid_argument("system index out of range");
    if (!initialized_) throw std::runtime_error("deaths before init");
    const System& y = sys_[s];
    deathtime.assign(deathtime_.begin() + y.start, deathtime_.begin() + y.start + y.n);
    dti.assign(dti_.begin() + y.start, dti_.begin() + y.start + y.n);
}

size_t Ensemble::alive(size_t s) const { return s < alive_.size() ? alive_[s] : 0; }
size_t Ensemble::count(size_t s) const { return s < sys_.size() ? sys_[s].r.size() : 0; }

}  // namespace glisser
