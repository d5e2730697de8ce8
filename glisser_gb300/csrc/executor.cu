// Block-loop executor.
//
// Data flow per time block (the reference's Executor::loop,
// src/executor.cu:598-764, without the SWIFT branch):
//   main stream : wait for this block's planet log upload -> time-block
//                 kernel over the alive particles (kill-encounter fused in its
//                 epilogue, flagged particles ballot-compacted into the
//                 hand-off list) -> stable 3-way partition into the second
//                 particle buffer -> counts and hand-off list to pinned host
//   host        : snapshot the planets, advance t, integrate the planets for
//                 the next block and upload that log on the copy stream into
//                 the other planet buffer -- or, with a planetary history,
//                 upload the interval's element tracks and evaluate every
//                 step's record on the device (interp.cu) -- overlapped with
//                 the kernel; then read the counts, stamp deathtimes and write
//                 encounter.out for the newly flagged particles.
// The full particle state comes back to the host mirror only when someone
// reads it (outputs, the C ABI), not every block; track snapshots are built
// on the device (track.cu).
#include "executor.h"
#include "interp.h"
#include "parallel.h"
#include "track.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <iomanip>
#include <numeric>
#include <sstream>

#include "timeblock.cuh"

namespace glisser {

int launch_partition(const glisser_particles* in, const glisser_particles* out, size_t n, void* scratch,
                     uint32_t* n0, uint32_t* n1, cudaStream_t stream);
size_t partition_scratch_bytes(size_t n);
int launch_copy_range(const glisser_particles* src, const glisser_particles* dst, size_t begin, size_t end,
                      cudaStream_t stream);
void* mlp_upload(const std::vector<uint8_t>& blob);
void mlp_free(void* dev);

namespace {

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

using clk = std::chrono::steady_clock;
double ms_since(clk::time_point a) { return std::chrono::duration<double, std::milli>(clk::now() - a).count(); }

struct DevParticles {
    glisser_particles p{};
    void* base = nullptr;
    void alloc(size_t n)
    {
        size_t cap = std::max<size_t>(n, 1);
        size_t bytes = cap * (9 * sizeof(double) + sizeof(uint16_t) + 2 * sizeof(uint32_t)) + 1024;
        ck(cudaMalloc(&base, bytes), "cudaMalloc particles");
        char* q = static_cast<char*>(base);
        double** dbl[9] = { &p.rx, &p.ry, &p.rz, &p.vx, &p.vy, &p.vz, &p.ax, &p.ay, &p.az };
        for (int k = 0; k < 9; k++) {
            *dbl[k] = reinterpret_cast<double*>(q);
            q += cap * sizeof(double);
        }
        p.deathtime_index = reinterpret_cast<uint32_t*>(q);
        q += cap * sizeof(uint32_t);
        p.id = reinterpret_cast<uint32_t*>(q);
        q += cap * sizeof(uint32_t);
        p.flags = reinterpret_cast<uint16_t*>(q);
    }
    void release()
    {
        if (base) cudaFree(base);
        base = nullptr;
    }
};

}  // namespace

struct Executor::Impl {
    cudaStream_t main = nullptr, htd = nullptr;
    cudaEvent_t start = nullptr, stop = nullptr, done = nullptr;
    cudaEvent_t uploaded[2] = { nullptr, nullptr };
    DevParticles buf[2];
    int cur = 0;
    // planet blocks (device + pinned staging)
    uint32_t log_cap = 0, max_npl = 0;
    double* d_log[2] = { nullptr, nullptr };
    double* d_m[2] = { nullptr, nullptr };
    double* d_rh[2] = { nullptr, nullptr };
    uint32_t* d_id[2] = { nullptr, nullptr };
    double* h_log[2] = { nullptr, nullptr };
    double* h_m[2] = { nullptr, nullptr };
    double* h_rh[2] = { nullptr, nullptr };
    uint32_t* h_id[2] = { nullptr, nullptr };
    uint32_t blk_npl[2] = { 0, 0 }, blk_len[2] = { 0, 0 };
    // device interpolation of the planetary history: element tracks per
    // buffer; log_on_device[b] = the host copy of log b is not filled
    InterpTrack* d_tracks[2] = { nullptr, nullptr };
    InterpTrack* h_tracks[2] = { nullptr, nullptr };
    bool log_on_device[2] = { false, false };
    // device track writer: bitmap/scan scratch, record staging, pinned copy
    uint32_t* d_track_scratch = nullptr;
    void* d_track_out = nullptr;
    void* h_track = nullptr;
    int blk = 1;   // planet buffer the next kernel uses (the first block fills 0)
    // hand-off and counters
    uint32_t* d_ctr = nullptr;            // [0] count [1] status [2] n0 [3] n1
    unsigned long long* d_evals = nullptr;
    uint32_t* h_ctr = nullptr;
    unsigned long long* h_evals = nullptr;
    uint32_t *d_ho_index = nullptr, *d_ho_id = nullptr, *d_ho_dti = nullptr;
    uint16_t* d_ho_flags = nullptr;
    uint32_t *h_ho_id = nullptr, *h_ho_dti = nullptr;
    uint16_t* h_ho_flags = nullptr;
    void* d_scratch = nullptr;
    // pinned download staging
    double* h_dl = nullptr;
    uint32_t* h_dl_u32 = nullptr;
    uint16_t* h_dl_flags = nullptr;
    void* d_mlp = nullptr;
    bool device = false;
    std::vector<double> host_store[2];    // planets-only runs keep the blocks here
    std::vector<uint32_t> host_ids[2];

    ~Impl()
    {
        if (!device) return;   // nothing was allocated on the device
        for (int b = 0; b < 2; b++) {
            buf[b].release();
            cudaFree(d_log[b]); cudaFree(d_m[b]); cudaFree(d_rh[b]); cudaFree(d_id[b]); cudaFree(d_tracks[b]);
            cudaFreeHost(h_tracks[b]);
            if (device) {
                cudaFreeHost(h_log[b]); cudaFreeHost(h_m[b]); cudaFreeHost(h_rh[b]); cudaFreeHost(h_id[b]);
            }
            if (uploaded[b]) cudaEventDestroy(uploaded[b]);
        }
        cudaFree(d_ctr); cudaFree(d_evals); cudaFree(d_ho_index); cudaFree(d_ho_id); cudaFree(d_ho_dti);
        cudaFree(d_ho_flags); cudaFree(d_scratch);
        cudaFreeHost(h_ctr); cudaFreeHost(h_evals); cudaFreeHost(h_ho_id); cudaFreeHost(h_ho_dti);
        cudaFreeHost(h_ho_flags); cudaFreeHost(h_dl); cudaFreeHost(h_dl_u32); cudaFreeHost(h_dl_flags);
        if (d_mlp) mlp_free(d_mlp);
        cudaFree(d_track_scratch); cudaFree(d_track_out); cudaFreeHost(h_track);
        if (start) cudaEventDestroy(start);
        if (stop) cudaEventDestroy(stop);
        if (done) cudaEventDestroy(done);
        if (main) cudaStreamDestroy(main);
        if (htd) cudaStreamDestroy(htd);
    }
};

Executor::Executor(const Config& c) : cfg(c), d_(new Impl()) {}
Executor::~Executor() = default;

void* Executor::stream() const { return d_->main; }

bool Executor::write_track_device(std::ostream& out, double* ms)
{
    Impl& d = *d_;
    if (!initialized_ || !d.device || !device_output_) return false;
    const size_t n = n_alive_host();
    if (max_id_ >= 0xFFFFFFE0u || (size_t)max_id_ > 4 * pa_.n + 4096) return false;   // sparse ids: host writer
    if (!d.d_track_out) {
        ck(cudaMalloc(&d.d_track_scratch, track_scratch_words(max_id_) * sizeof(uint32_t)), "cudaMalloc track scratch");
        ck(cudaMalloc(&d.d_track_out, std::max<size_t>(pa_.n, 1) * 28), "cudaMalloc track records");
        ck(cudaMallocHost(&d.h_track, std::max<size_t>(pa_.n, 1) * 28), "pinned track records");
    }
    const Planets& pl = snapshot_;
    double cm;
    Vec3 cr, cv;
    track_particle_frame(pl, cfg.write_bary_track, cm, cr, cv);
    TrackFrame fr{ cm, { cr.x, cr.y, cr.z }, { cv.x, cv.y, cv.z } };
    ck(cudaEventRecord(d.start, d.main), "event");
    ck(launch_track_records(&d.buf[d.cur].p, (uint32_t)n, max_id_, fr, d.d_track_scratch, d.d_track_out, d.main),
       "track kernels");
    launches_total_ += 4;
    ck(cudaMemcpyAsync(d.h_track, d.d_track_out, n * 28, cudaMemcpyDeviceToHost, d.main), "track download");
    ck(cudaEventRecord(d.stop, d.main), "event");
    ck(cudaEventSynchronize(d.stop), "track");
    if (ms) {
        float f = 0;
        ck(cudaEventElapsedTime(&f, d.start, d.stop), "elapsed");
        *ms = f;
    }
    write_track_planets(out, pl, t, cfg.write_bary_track);
    uint64_t cnt = n;
    out.write(reinterpret_cast<const char*>(&cnt), sizeof cnt);
    out.write(static_cast<const char*>(d.h_track), (std::streamsize)(n * 28));
    out.flush();
    return true;
}

void Executor::set_deathtime(uint32_t id, double t)
{
    if (dt_dense_on_ && id < dt_dense_.size()) dt_dense_[id] = t;
    else deathtime_[id] = t;
}

double Executor::get_deathtime(uint32_t id) const
{
    if (dt_dense_on_ && id < dt_dense_.size()) return dt_dense_[id];
    auto it = deathtime_.find(id);
    return it == deathtime_.end() ? 0.0 : it->second;
}

void Executor::device_view(glisser_particles* pa, size_t* n, double* dt, double* mu) const
{
    if (!initialized_) throw std::invalid_argument("device_view: call init first");
    if (!d_->device) {
        *pa = glisser_particles{};
        *n = 0;
    } else {
        *pa = d_->buf[d_->cur].p;
        *n = n_dev_;
    }
    *dt = cur_dt_;
    *mu = pl_.m[0];
}

void Executor::load()
{
    load_state(cfg, pl_, pa_);
    for (size_t k = 0; k < pa_.n; k++) set_deathtime(pa_.id[k], pa_.deathtime[k]);
    loaded_pl_ = loaded_pa_ = true;
    t = cfg.t_0;
}

void Executor::set_planets(size_t n, const double* m, const double* r, const double* v, const uint32_t* id)
{
    if (initialized_) throw std::runtime_error("planets can only be set before init");
    pl_.resize(n);
    pl_.n_alive = n;
    for (size_t i = 0; i < n; i++) {
        pl_.m[i] = m[i] * cfg.big_g;
        pl_.r[i] = Vec3{ r[3 * i], r[3 * i + 1], r[3 * i + 2] };
        pl_.v[i] = Vec3{ v[3 * i], v[3 * i + 1], v[3 * i + 2] };
        if (cfg.readmomenta) pl_.v[i] = pl_.v[i] / m[i];
        pl_.id[i] = id ? id[i] : (uint32_t)i;
    }
    loaded_pl_ = true;
    t = cfg.t_0;
}

void Executor::set_particles(size_t n, const double* r, const double* v, const uint32_t* id, const uint16_t* flags,
                             const double* deathtime)
{
    if (!initialized_) {
        n = std::min(n, (size_t)cfg.max_particle);
        pa_.resize(n);
        for (size_t k = 0; k < n; k++) {
            pa_.r[k] = Vec3{ r[3 * k], r[3 * k + 1], r[3 * k + 2] };
            pa_.v[k] = Vec3{ v[3 * k], v[3 * k + 1], v[3 * k + 2] };
            pa_.id[k] = id ? id[k] : (uint32_t)k;
            pa_.flags[k] = flags ? flags[k] : 0;
            pa_.deathtime[k] = deathtime ? deathtime[k] : 0.0;
            set_deathtime(pa_.id[k], pa_.deathtime[k]);
        }
        loaded_pa_ = true;
        return;
    }
    // after init: overwrite the state of the n particles in device order
    // (same ids, same order as glisser_get_particles returns them)
    if (n != pa_.n) throw std::runtime_error("set_particles after init must pass every particle");
    if (!d_->device || n == 0) return;
    // positions, velocities (and flags) through the pinned staging buffer;
    // ids and the carried accelerations stay on the device
    Impl& d = *d_;
    double* st = d.h_dl;
    parallel_for(n, [&](size_t b, size_t e) {
        for (size_t k = b; k < e; k++) {
            st[k] = r[3 * k]; st[n + k] = r[3 * k + 1]; st[2 * n + k] = r[3 * k + 2];
            st[3 * n + k] = v[3 * k]; st[4 * n + k] = v[3 * k + 1]; st[5 * n + k] = v[3 * k + 2];
        }
    });
    glisser_particles& p = d.buf[d.cur].p;
    glisser_particles& q = d.buf[d.cur ^ 1].p;
    double* dst[6] = { p.rx, p.ry, p.rz, p.vx, p.vy, p.vz };
    double* mir[6] = { q.rx, q.ry, q.rz, q.vx, q.vy, q.vz };
    for (int c = 0; c < 6; c++) {
        ck(cudaMemcpyAsync(dst[c], st + c * n, n * sizeof(double), cudaMemcpyHostToDevice, d.main), "upload state");
        ck(cudaMemcpyAsync(mir[c], dst[c], n * sizeof(double), cudaMemcpyDeviceToDevice, d.main), "mirror state");
    }
    if (flags) {
        std::memcpy(d.h_dl_flags, flags, n * sizeof(uint16_t));
        ck(cudaMemcpyAsync(p.flags, d.h_dl_flags, n * sizeof(uint16_t), cudaMemcpyHostToDevice, d.main), "upload flags");
        ck(cudaMemcpyAsync(q.flags, p.flags, n * sizeof(uint16_t), cudaMemcpyDeviceToDevice, d.main), "mirror flags");
    }
    ck(cudaStreamSynchronize(d.main), "upload sync");
    host_dirty_ = true;
}

void Executor::set_starter(int starter, const std::vector<uint8_t>* blob)
{
    if (starter < GLISSER_STARTER_CLASSIC || starter > GLISSER_STARTER_LEARNED)
        throw std::runtime_error("unknown starter");
    if (starter == GLISSER_STARTER_LEARNED) {
        if (!blob) throw std::runtime_error("the learned starter needs weights");
        if (d_->d_mlp) mlp_free(d_->d_mlp);
        d_->d_mlp = mlp_upload(*blob);
    }
    starter_ = starter;
}

// helio_acc_particle<old=true> at the first step (src/wh.cpp:611-657): the
// CPU flag convention (last planet wins, planet index in the high byte).
void Executor::initial_accelerations(std::vector<Vec3>& acc)
{
    Vec3 h0 = integ_.accelerations(pl_);
    size_t npl = pl_.n_alive;
    acc.assign(pa_.n, h0);
    for (size_t k = 0; k < pa_.n; k++) {
        Vec3 a = h0;
        for (size_t j = 1; j < npl; j++) {
            Vec3 dr = pa_.r[k] - pl_.r[j];
            double r2 = dr.lensq();
            double irij3 = 1. / (r2 * std::sqrt(r2));
            a -= dr * (pl_.m[j] * irij3);
            if (r2 < rh_[j] * rh_[j]) {
                set_deathtime(pa_.id[k], 0);   // the reference stamps time 0 here
                pa_.flags[k] = (uint16_t)((j << 8) | 0x0001);
            }
        }
        double r2 = pa_.r[k].lensq();
        if (r2 < rh_[0] * rh_[0]) {
            set_deathtime(pa_.id[k], 0);
            pa_.flags[k] = 0x0001;
        }
        if (r2 > cfg.outer_radius * cfg.outer_radius) {
            set_deathtime(pa_.id[k], 0);
            pa_.flags[k] = 0x0002;
        }
        acc[k] = a;
    }
}

void Executor::upload_particles(const std::vector<Vec3>& acc)
{
    size_t n = pa_.n;
    std::vector<double> col(n);
    auto up = [&](double* dst, auto get) {
        for (size_t k = 0; k < n; k++) col[k] = get(k);
        ck(cudaMemcpy(dst, col.data(), n * sizeof(double), cudaMemcpyHostToDevice), "upload particles");
    };
    for (int b = 0; b < 2; b++) {
        glisser_particles& p = d_->buf[b].p;
        up(p.rx, [&](size_t k) { return pa_.r[k].x; });
        up(p.ry, [&](size_t k) { return pa_.r[k].y; });
        up(p.rz, [&](size_t k) { return pa_.r[k].z; });
        up(p.vx, [&](size_t k) { return pa_.v[k].x; });
        up(p.vy, [&](size_t k) { return pa_.v[k].y; });
        up(p.vz, [&](size_t k) { return pa_.v[k].z; });
        up(p.ax, [&](size_t k) { return acc[k].x; });
        up(p.ay, [&](size_t k) { return acc[k].y; });
        up(p.az, [&](size_t k) { return acc[k].z; });
        ck(cudaMemcpy(p.flags, pa_.flags.data(), n * sizeof(uint16_t), cudaMemcpyHostToDevice), "upload flags");
        ck(cudaMemcpy(p.id, pa_.id.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload ids");
        ck(cudaMemcpy(p.deathtime_index, pa_.deathtime_index.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice),
           "upload deathtime index");
    }
    host_dirty_ = false;
}

void Executor::download_particles()
{
    if (!host_dirty_ || !initialized_) return;
    size_t n = pa_.n;
    Impl& d = *d_;
    glisser_particles& p = d.buf[d.cur].p;
    double* src[6] = { p.rx, p.ry, p.rz, p.vx, p.vy, p.vz };
    for (int k = 0; k < 6; k++)
        ck(cudaMemcpyAsync(d.h_dl + k * n, src[k], n * sizeof(double), cudaMemcpyDeviceToHost, d.main), "download");
    ck(cudaMemcpyAsync(d.h_dl_u32, p.id, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.main), "download ids");
    ck(cudaMemcpyAsync(d.h_dl_u32 + n, p.deathtime_index, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.main),
       "download deathtime index");
    ck(cudaMemcpyAsync(d.h_dl_flags, p.flags, n * sizeof(uint16_t), cudaMemcpyDeviceToHost, d.main), "download flags");
    ck(cudaStreamSynchronize(d.main), "download sync");
    parallel_for(n, [&](size_t b, size_t e) {
        for (size_t k = b; k < e; k++) {
            pa_.r[k] = Vec3{ d.h_dl[k], d.h_dl[n + k], d.h_dl[2 * n + k] };
            pa_.v[k] = Vec3{ d.h_dl[3 * n + k], d.h_dl[4 * n + k], d.h_dl[5 * n + k] };
            pa_.id[k] = d.h_dl_u32[k];
            pa_.deathtime_index[k] = d.h_dl_u32[n + k];
            pa_.flags[k] = d.h_dl_flags[k];
            pa_.deathtime[k] = get_deathtime(pa_.id[k]);
        }
    });
    host_dirty_ = false;
}

const Particles& Executor::particles()
{
    download_particles();
    return pa_;
}

void Executor::update_planets()
{
    prev_dt_ = cur_dt_;
    prev_tbsize_ = cur_tbsize_;
    integ_.encounter_radii(pl_, cfg.cull_radius, cfg.encounter_sphere_factor, rh_);
    Impl& d = *d_;
    const int nb = d.blk ^ 1;   // the planet buffer the running kernel is not reading
    double* log = d.h_log[nb];
    uint32_t npl;
    if (cfg.interp_planets) {
        auto& ip = interp_;
        if (ip.cur_ts == ip.n_ts) {
            ip.next(pl_);
            ip.cur_ts = 0;
            t = ip.t0;
            starting_interval_ = true;
        } else {
            starting_interval_ = ip.cur_ts == 0;
        }
        cur_dt_ = ip.eff_dt;
        cur_tbsize_ = std::min<size_t>(cfg.tbsize, ip.n_ts - ip.cur_ts);
        npl = (uint32_t)(ip.n_alive + 1);
        if (npl > d.max_npl) throw StateError("planetary history has more planets than the device buffers hold");
        if (d.device && device_interp_) {
            // the device evaluates every step's record (interp.cu); the host
            // keeps the interval bookkeeping and the live planets, which end
            // at the block's last step time (accumulated as the per-step
            // fill accumulates it)
            for (size_t j = 0; j < ip.n_alive; j++) {
                pl_.id[j + 1] = ip.ids[j];
                pl_.m[j + 1] = ip.mass[j];
                InterpTrack& q = d.h_tracks[nb][j];
                const Vec3* src[4] = { &ip.aei_i[j], &ip.daei[j], &ip.oom_i[j], &ip.doom[j] };
                double* dst[4] = { q.aei_i, q.daei, q.oom_i, q.doom };
                for (int c = 0; c < 4; c++) {
                    dst[c][0] = src[c]->x;
                    dst[c][1] = src[c]->y;
                    dst[c][2] = src[c]->z;
                }
                q.m = ip.mass[j];
                q.pad = 0;
            }
            double tt = ip.rel_t + cur_dt_, last = tt;
            for (size_t k = 0; k < cur_tbsize_; k++) {
                if (tt > ip.t1 - ip.t0 + 1e-8)
                    throw std::runtime_error("interpolation ran too long, timechunk exceeded lookup boundary");
                last = tt;
                tt += cur_dt_;
            }
            if (cur_tbsize_ > 0) {
                pl_.r[0] = pl_.v[0] = Vec3{ 0, 0, 0 };
                ip.fill_one(pl_, last);
            }
            ck(cudaMemcpyAsync(d.d_tracks[nb], d.h_tracks[nb], ip.n_alive * sizeof(InterpTrack),
                               cudaMemcpyHostToDevice, d.htd), "upload tracks");
            ck(launch_interp_fill(d.d_tracks[nb], npl - 1, (uint32_t)cur_tbsize_, ip.rel_t, cur_dt_, d.d_log[nb],
                                  d.htd), "interpolation kernel");
            launches_total_ += 1;
            d.log_on_device[nb] = true;
        } else {
            // positions into the log records (after the h0 slot), then h0
            ip.fill(pl_, cur_tbsize_, ip.rel_t, cur_dt_, log + 3, 3 * (size_t)npl);
            for (size_t s = 0; s < cur_tbsize_; s++) {
                double* rec = log + s * 3 * npl;
                Vec3 h0 = indirect_term(rec + 3, pl_.m, npl);
                rec[0] = h0.x; rec[1] = h0.y; rec[2] = h0.z;
            }
            d.log_on_device[nb] = false;
        }
        pl_.n_alive = npl;
        ip.rel_t += (double)cur_tbsize_ * cur_dt_;
        ip.cur_ts += cur_tbsize_;
    } else {
        cur_dt_ = cfg.dt;
        cur_tbsize_ = cfg.tbsize;
        npl = (uint32_t)pl_.n_alive;
        d.log_on_device[nb] = false;
        for (size_t s = 0; s < cur_tbsize_; s++) {
            Vec3 h0 = integ_.step(pl_, cur_dt_);
            double* rec = log + s * 3 * npl;
            rec[0] = h0.x; rec[1] = h0.y; rec[2] = h0.z;
            for (uint32_t j = 1; j < npl; j++) {
                rec[3 * j] = pl_.r[j].x;
                rec[3 * j + 1] = pl_.r[j].y;
                rec[3 * j + 2] = pl_.r[j].z;
            }
        }
    }
    for (uint32_t j = 0; j < npl; j++) {
        d.h_m[nb][j] = pl_.m[j];
        d.h_id[nb][j] = pl_.id[j];
        d.h_rh[nb][j] = rh_[j];
    }
    d.blk_npl[nb] = npl;
    d.blk_len[nb] = (uint32_t)cur_tbsize_;
    d.blk = nb;
    if (!d.device) return;
    size_t recs = (cur_tbsize_ + 1) & ~(size_t)1;
    if (!d.log_on_device[nb])
        ck(cudaMemcpyAsync(d.d_log[nb], log, recs * 3 * npl * sizeof(double), cudaMemcpyHostToDevice, d.htd),
           "upload log");
    ck(cudaMemcpyAsync(d.d_m[nb], d.h_m[nb], npl * sizeof(double), cudaMemcpyHostToDevice, d.htd), "upload m");
    ck(cudaMemcpyAsync(d.d_id[nb], d.h_id[nb], npl * sizeof(uint32_t), cudaMemcpyHostToDevice, d.htd), "upload ids");
    ck(cudaMemcpyAsync(d.d_rh[nb], d.h_rh[nb], npl * sizeof(double), cudaMemcpyHostToDevice, d.htd), "upload rh");
    ck(cudaEventRecord(d.uploaded[nb], d.htd), "record upload");
}

void Executor::planet_block(std::vector<double>& log, std::vector<double>& m, std::vector<uint32_t>& id,
                            std::vector<double>& rh, uint32_t& npl, uint32_t& len) const
{
    Impl& d = *d_;
    int b = d.blk;
    npl = d.blk_npl[b];
    len = d.blk_len[b];
    if (d.log_on_device[b] && len > 0) {
        ck(cudaEventSynchronize(d.uploaded[b]), "interpolation");
        ck(cudaMemcpy(d.h_log[b], d.d_log[b], (size_t)len * 3 * npl * sizeof(double), cudaMemcpyDeviceToHost),
           "download log");
    }
    log.assign(d.h_log[b], d.h_log[b] + (size_t)len * 3 * npl);
    m.assign(d.h_m[b], d.h_m[b] + npl);
    rh.assign(d.h_rh[b], d.h_rh[b] + npl);
    id.assign(d.h_id[b], d.h_id[b] + npl);
}

void Executor::init()
{
    if (!loaded_pl_ || !loaded_pa_) throw std::runtime_error("init before the state was loaded");
    if (initialized_) throw std::runtime_error("init called twice");
    Impl& d = *d_;
    // glisse only supports heliocentric coordinates (src/executor.cu:90-91)
    Vec3 r0 = pl_.r[0], v0 = pl_.v[0];
    for (size_t i = 0; i < pl_.n; i++) {
        pl_.r[i] -= r0;
        pl_.v[i] -= v0;
    }
    for (size_t k = 0; k < pa_.n; k++) {
        pa_.r[k] -= r0;
        pa_.v[k] -= v0;
    }
    if (cfg.interp_planets) {
        auto& ip = interp_;
        ip.open(cfg.planet_history_file, cfg.interp_maxpl, cfg.dt, t, pl_);
        while (ip.t1 <= t) ip.next(pl_);
        if (std::isinf(ip.t0)) throw std::runtime_error("lookup file starts past the given Initial-Time");
        ip.cur_ts = 0;
        ip.n_ts = std::max<size_t>(1, (size_t)std::round((ip.t1 - t) / cfg.dt));
        ip.eff_dt = (ip.t1 - t) / (double)ip.n_ts;
        ip.rel_t = t - ip.t0;
        ip.fill_one(pl_, ip.rel_t);
        pl_.n_alive = ip.n_alive + 1;
    }
    integ_.init(pl_);
    integ_.encounter_radii(pl_, cfg.cull_radius, cfg.encounter_sphere_factor, rh_);
    std::vector<Vec3> acc;
    initial_accelerations(acc);

    // initial planet energy (calculate_planet_metrics, src/wh.cpp:422-470)
    {
        size_t n = pl_.n_alive;
        double M = 0;
        Vec3 br{ 0, 0, 0 }, bv{ 0, 0, 0 };
        for (size_t i = 0; i < n; i++) {
            br += pl_.r[i] * pl_.m[i];
            bv += pl_.v[i] * pl_.m[i];
            M += pl_.m[i];
        }
        br = br / M;
        bv = bv / M;
        double ke = 0, pe = 0;
        for (size_t i = 0; i < n; i++) ke += 0.5 * (pl_.v[i] - bv).lensq() * pl_.m[i];
        for (size_t i = 0; i + 1 < n; i++)
            for (size_t j = i + 1; j < n; j++) pe -= pl_.m[i] * pl_.m[j] / std::sqrt((pl_.r[i] - pl_.r[j]).lensq());
        e0 = ke + pe;
    }

    // alive first, then encounter particles; accelerations travel with their
    // particles (the reference leaves them in load order)
    std::vector<size_t> order(pa_.n);
    std::iota(order.begin(), order.end(), 0);
    auto mid = std::stable_partition(order.begin(), order.end(), [&](size_t k) { return pa_.flags[k] == 0; });
    size_t n_unflagged = (size_t)(mid - order.begin());
    auto mid2 = std::stable_partition(mid, order.end(), [&](size_t k) { return (pa_.flags[k] & 0xFE) == 0; });
    size_t n_alive = (size_t)(mid2 - order.begin());
    {
        Particles q;
        q.resize(pa_.n);
        std::vector<Vec3> a2(pa_.n);
        for (size_t k = 0; k < pa_.n; k++) {
            size_t s = order[k];
            q.r[k] = pa_.r[s]; q.v[k] = pa_.v[s]; q.id[k] = pa_.id[s]; q.flags[k] = pa_.flags[s];
            q.deathtime[k] = pa_.deathtime[s]; q.deathtime_index[k] = pa_.deathtime_index[s];
            a2[k] = acc[s];
        }
        pa_ = std::move(q);
        acc.swap(a2);
    }
    (void)n_unflagged;

    max_id_ = 0;
    for (size_t k = 0; k < pa_.n; k++) max_id_ = std::max(max_id_, pa_.id[k]);
    // dense ids: deathtimes in a vector indexed by id (the per-download lookup
    // is then a load, not a hash probe)
    if ((size_t)max_id_ <= 4 * pa_.n + 4096) {
        dt_dense_.assign((size_t)max_id_ + 1, 0.0);
        for (const auto& e : deathtime_)
            if (e.first <= max_id_) dt_dense_[e.first] = e.second;
        deathtime_.clear();
        dt_dense_on_ = true;
    }
    d.max_npl = (uint32_t)std::min<size_t>(pl_.n, MAX_PLANETS);
    if (pl_.n > (size_t)MAX_PLANETS) throw StateError("more than 64 planets");
    d.log_cap = (cfg.tbsize + 1u) & ~1u;
    size_t log_bytes = (size_t)d.log_cap * 3 * d.max_npl * sizeof(double);
    size_t n = pa_.n;
    d.device = n > 0;
    if (!d.device) {
        // planets-only run (Limit-Particle-Count 0): no device work at all
        for (int b = 0; b < 2; b++) {
            d.host_store[b].assign(log_bytes / sizeof(double) + 3 * (size_t)d.max_npl, 0.0);
            d.host_ids[b].assign(d.max_npl, 0);
            d.h_log[b] = d.host_store[b].data();
            d.h_m[b] = d.h_log[b] + log_bytes / sizeof(double);
            d.h_rh[b] = d.h_m[b] + d.max_npl;
            d.h_id[b] = d.host_ids[b].data();
        }
        n_dev_ = 0;
        n_encounter_ = 0;
        snapshot_ = pl_;
        initialized_ = true;
        update_planets();
        return;
    }
    // device resources
    ck(cudaStreamCreateWithFlags(&d.main, cudaStreamNonBlocking), "stream");
    ck(cudaStreamCreateWithFlags(&d.htd, cudaStreamNonBlocking), "stream");
    ck(cudaEventCreate(&d.start), "event");
    ck(cudaEventCreate(&d.stop), "event");
    ck(cudaEventCreateWithFlags(&d.done, cudaEventDisableTiming), "event");
    for (int b = 0; b < 2; b++) {
        d.buf[b].alloc(n);
        ck(cudaEventCreateWithFlags(&d.uploaded[b], cudaEventDisableTiming), "event");
    }
    for (int b = 0; b < 2; b++) {
        ck(cudaMalloc(&d.d_log[b], log_bytes), "cudaMalloc log");
        ck(cudaMemset(d.d_log[b], 0, log_bytes), "memset log");
        ck(cudaMalloc(&d.d_m[b], d.max_npl * sizeof(double)), "cudaMalloc m");
        ck(cudaMalloc(&d.d_rh[b], d.max_npl * sizeof(double)), "cudaMalloc rh");
        ck(cudaMalloc(&d.d_id[b], d.max_npl * sizeof(uint32_t)), "cudaMalloc id");
        ck(cudaMallocHost(&d.h_log[b], log_bytes), "cudaMallocHost log");
        std::memset(d.h_log[b], 0, log_bytes);
        ck(cudaMallocHost(&d.h_m[b], d.max_npl * sizeof(double)), "pinned");
        ck(cudaMallocHost(&d.h_rh[b], d.max_npl * sizeof(double)), "pinned");
        ck(cudaMallocHost(&d.h_id[b], d.max_npl * sizeof(uint32_t)), "pinned");
        ck(cudaMalloc(&d.d_tracks[b], d.max_npl * sizeof(InterpTrack)), "cudaMalloc tracks");
        ck(cudaMallocHost(&d.h_tracks[b], d.max_npl * sizeof(InterpTrack)), "pinned");
    }
    size_t cap = std::max<size_t>(n, 1);
    ck(cudaMalloc(&d.d_ctr, 16 * sizeof(uint32_t)), "cudaMalloc counters");
    ck(cudaMalloc(&d.d_evals, sizeof(unsigned long long)), "cudaMalloc evals");
    ck(cudaMallocHost(&d.h_ctr, 16 * sizeof(uint32_t)), "pinned");
    ck(cudaMallocHost(&d.h_evals, sizeof(unsigned long long)), "pinned");
    ck(cudaMalloc(&d.d_ho_index, cap * sizeof(uint32_t)), "cudaMalloc hand-off");
    ck(cudaMalloc(&d.d_ho_id, cap * sizeof(uint32_t)), "cudaMalloc hand-off");
    ck(cudaMalloc(&d.d_ho_dti, cap * sizeof(uint32_t)), "cudaMalloc hand-off");
    ck(cudaMalloc(&d.d_ho_flags, cap * sizeof(uint16_t)), "cudaMalloc hand-off");
    ck(cudaMallocHost(&d.h_ho_id, cap * sizeof(uint32_t)), "pinned");
    ck(cudaMallocHost(&d.h_ho_dti, cap * sizeof(uint32_t)), "pinned");
    ck(cudaMallocHost(&d.h_ho_flags, cap * sizeof(uint16_t)), "pinned");
    ck(cudaMalloc(&d.d_scratch, partition_scratch_bytes(cap)), "cudaMalloc scratch");
    ck(cudaMallocHost(&d.h_dl, cap * 6 * sizeof(double)), "pinned");
    ck(cudaMallocHost(&d.h_dl_u32, cap * 2 * sizeof(uint32_t)), "pinned");
    ck(cudaMallocHost(&d.h_dl_flags, cap * sizeof(uint16_t)), "pinned");
    upload_particles(acc);
    n_dev_ = n_alive;
    n_encounter_ = 0;
    snapshot_ = pl_;
    initialized_ = true;
    update_planets();
    if (log) {
        *log << std::setprecision(7);
        *log << "e_0 (planets) = " << e0 << std::endl;
        *log << "n_particle = " << pa_.n << std::endl;
        *log << "n_particle_alive = " << n_alive << std::endl;
        *log << "==================================" << std::endl;
        *log << "Sending initial conditions to GPU." << std::endl;
        *log << "       Starting simulation.       " << std::endl << std::endl;
    }
}

bool Executor::step_block(double* cpu_ms, double* gpu_ms)
{
    if (!initialized_) throw std::runtime_error("step before init");
    Impl& d = *d_;
    const int used = d.blk;
    const size_t prev_alive = n_dev_;
    float gpu = 0;
    if (n_dev_ > 0) {
        ck(cudaStreamWaitEvent(d.main, d.uploaded[used], 0), "wait upload");
        ck(cudaMemsetAsync(d.d_ctr, 0, 16 * sizeof(uint32_t), d.main), "memset counters");
        ck(cudaMemsetAsync(d.d_evals, 0, sizeof(unsigned long long), d.main), "memset evals");
        glisser_planet_block pb{};
        pb.log = d.d_log[used];
        pb.m = d.d_m[used];
        pb.id = d.d_id[used];
        pb.rh = d.d_rh[used];
        pb.npl = d.blk_npl[used];
        pb.len = d.blk_len[used];
        pb.capacity = d.log_cap;
        glisser_step_params sp{};
        sp.dt = cur_dt_;
        sp.outer_radius = cfg.outer_radius;
        sp.starter = starter_;
        sp.kill_encounters = cfg.resolve_encounters ? 0 : 1;
        sp.mlp = starter_ == GLISSER_STARTER_LEARNED ? d.d_mlp : nullptr;
        sp.kepler_tol = kepler_tol_;
        glisser_handoff ho{};
        ho.count = d.d_ctr;
        ho.status = d.d_ctr + 1;
        ho.index = d.d_ho_index;
        ho.id = d.d_ho_id;
        ho.flags = d.d_ho_flags;
        ho.deathtime_index = d.d_ho_dti;
        ho.capacity = (uint32_t)std::max<size_t>(pa_.n, 1);
        ho.evals = d.d_evals;
        ck(cudaEventRecord(d.start, d.main), "event");
        int rc = launch_timeblock(&d.buf[d.cur].p, n_dev_, &pb, &sp, &ho, d.main);
        if (rc != GLISSER_OK) throw CudaError(std::string("time-block launch failed: ") + timeblock_error());
        ck(cudaEventRecord(d.stop, d.main), "event");
        int nxt = d.cur ^ 1;
        rc = launch_partition(&d.buf[d.cur].p, &d.buf[nxt].p, n_dev_, d.d_scratch, d.d_ctr + 2, d.d_ctr + 3, d.main);
        launches_total_ += 4;   // time block + count, scan, scatter
        if (rc != GLISSER_OK) throw CudaError("partition launch failed");
        ck(cudaMemcpyAsync(d.h_ctr, d.d_ctr, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.main), "counters");
        ck(cudaMemcpyAsync(d.h_evals, d.d_evals, sizeof(unsigned long long), cudaMemcpyDeviceToHost, d.main), "evals");
        ck(cudaEventRecord(d.done, d.main), "event");
        d.cur = nxt;
        host_dirty_ = true;
    }
    // host work overlapped with the kernel
    auto c0 = clk::now();
    snapshot_ = pl_;
    t += cur_dt_ * (double)cur_tbsize_;
    update_planets();
    double cpu = ms_since(c0);
    if (prev_alive > 0) {
        ck(cudaEventSynchronize(d.done), "block");
        ck(cudaEventElapsedTime(&gpu, d.start, d.stop), "elapsed");
        uint32_t status = d.h_ctr[1];
        if (status) throw CudaError("time-block kernel reported a planet-log staging timeout");
        uint32_t n0 = d.h_ctr[2], n1 = d.h_ctr[3];
        uint32_t k = std::min<uint32_t>(d.h_ctr[0], (uint32_t)std::max<size_t>(pa_.n, 1));
        evals_total_ += *d.h_evals;
        // both particle buffers must agree on the particles that left the
        // alive range this block (the next partition reads only the alive one)
        if (n0 + n1 < prev_alive) {
            int rc = launch_copy_range(&d.buf[d.cur].p, &d.buf[d.cur ^ 1].p, n0 + n1, prev_alive, d.main);
            if (rc != GLISSER_OK) throw CudaError("copy launch failed");
            launches_total_ += 1;
        }
        // particles that kept their flags advanced the whole block; the
        // flagged ones add their deathtime index below
        psteps_total_ += (unsigned long long)(prev_alive - std::min<size_t>(prev_alive, d.h_ctr[0])) *
                         d.blk_len[used];
        n_dev_ = cfg.resolve_encounters ? n0 : n0 + n1;
        n_encounter_ = cfg.resolve_encounters ? n1 : 0;
        flagged_.clear();
        if (k) {
            ck(cudaMemcpyAsync(d.h_ho_id, d.d_ho_id, k * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.main), "hand-off");
            ck(cudaMemcpyAsync(d.h_ho_dti, d.d_ho_dti, k * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.main), "hand-off");
            ck(cudaMemcpyAsync(d.h_ho_flags, d.d_ho_flags, k * sizeof(uint16_t), cudaMemcpyDeviceToHost, d.main),
               "hand-off");
            ck(cudaStreamSynchronize(d.main), "hand-off sync");
            for (uint32_t q = 0; q < k; q++) {
                flagged_.push_back({ d.h_ho_id[q], d.h_ho_flags[q], d.h_ho_dti[q] });
                psteps_total_ += d.h_ho_dti[q];
            }
            std::sort(flagged_.begin(), flagged_.end(),
                      [](const FlaggedEntry& a, const FlaggedEntry& b) { return a.id < b.id; });
            float tf = (float)t;
            for (auto& f : flagged_) {
                set_deathtime(f.id, tf);
                if ((f.flags & 0x04) && log)
                    *log << "warning - particle " << f.id << " did not converge on GPU" << std::endl;
                if (encounter_out) {
                    *encounter_out << std::setprecision(17) << f.id << ((f.flags & 0x80) ? " death " : " encounter ")
                                   << t << "\n";
                }
            }
        }
    }
    if (cpu_ms) *cpu_ms = cpu;
    if (gpu_ms) *gpu_ms = gpu;
    return starting_interval_ || !cfg.resolve_encounters;
}

void Executor::finish()
{
    if (initialized_ && d_->device) {
        ck(cudaStreamSynchronize(d_->main), "finish");
        download_particles();
    }
    if (log) *log << "Simulation finished. t = " << t << ". n_particle = " << n_alive_host() << std::endl;
}

}  // namespace glisser
