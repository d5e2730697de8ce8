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
    cudaStream_t main = nullptr, htd = nullptr, dth = nullptr;
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
        if (dth) cudaStreamDestroy(dth);
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
    net_next_ = true;
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
    initial_flagged_.clear();
    if (cfg.resolve_encounters)
        for (size_t k = n_unflagged; k < n_alive; k++) initial_flagged_.push_back({ pa_.id[k], pa_.flags[k], 0 });
    if (cfg.resolve_encounters)
        swift_.reset(new SwiftRunner(cfg.swift_path, cfg.outfolder.empty() ? std::string(".") : cfg.outfolder,
                                     cfg.swift_statlen, cfg.swift_part_min, cfg.num_swift, cfg.outer_radius));

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
        if (timing_out) write_timing_header();
        return;
    }
    // device resources
    ck(cudaStreamCreateWithFlags(&d.main, cudaStreamNonBlocking), "stream");
    ck(cudaStreamCreateWithFlags(&d.htd, cudaStreamNonBlocking), "stream");
    ck(cudaStreamCreateWithFlags(&d.dth, cudaStreamNonBlocking), "stream");
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
    ck(cudaMalloc(&d.d_evals, 4 * sizeof(unsigned long long)), "cudaMalloc evals");
    ck(cudaMallocHost(&d.h_ctr, 16 * sizeof(uint32_t)), "pinned");
    ck(cudaMallocHost(&d.h_evals, 4 * sizeof(unsigned long long)), "pinned");
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
    if (timing_out) write_timing_header();
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
    const auto t_total = clk::now();
    BlockTiming tm;
    const int used = d.blk;
    const bool resolve = cfg.resolve_encounters && d.device;
    // the kernel integrates the unflagged particles; with Resolve-Encounters
    // the encounter particles that follow them are resumed on SWIFT over the
    // same block and rejoin at the partition after it
    const size_t n_kernel = n_dev_;
    const size_t n_enc = resolve ? n_encounter_ : 0;
    const size_t n_range = n_kernel + n_enc;
    const size_t n_enc_start = n_encounter_;
    float gpu = 0;
    bool partitioned = false;
    auto launch_partition_now = [&]() {
        int nxt = d.cur ^ 1;
        int rc = launch_partition(&d.buf[d.cur].p, &d.buf[nxt].p, n_range, d.d_scratch, d.d_ctr + 2, d.d_ctr + 3,
                                  d.main);
        launches_total_ += 3;   // count, scan, scatter
        if (rc != GLISSER_OK) throw CudaError("partition launch failed");
        ck(cudaMemcpyAsync(d.h_ctr, d.d_ctr, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.main), "counters");
        ck(cudaMemcpyAsync(d.h_evals, d.d_evals, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, d.main),
           "evals");
        ck(cudaEventRecord(d.done, d.main), "event");
        d.cur = nxt;
        host_dirty_ = true;
        partitioned = true;
    };
    if (n_range > 0) {
        ck(cudaMemsetAsync(d.d_ctr, 0, 16 * sizeof(uint32_t), d.main), "memset counters");
        ck(cudaMemsetAsync(d.d_evals, 0, 4 * sizeof(unsigned long long), d.main), "memset evals");
    }
    if (n_kernel > 0) {
        ck(cudaStreamWaitEvent(d.main, d.uploaded[used], 0), "wait upload");
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
        const bool net = starter_ == GLISSER_STARTER_LEARNED && net_next_;
        sp.starter = starter_ == GLISSER_STARTER_LEARNED && !net ? GLISSER_STARTER_SERIES : starter_;
        sp.kill_encounters = cfg.resolve_encounters ? GLISSER_ENCOUNTERS_ROLLBACK : GLISSER_ENCOUNTERS_KILL;
        sp.mlp = net ? d.d_mlp : nullptr;
        net_blocks_ += net;
        sp.kepler_tol = kepler_tol_;
        sp.kick = kick_;
        glisser_handoff ho{};
        ho.count = d.d_ctr;
        ho.status = d.d_ctr + 1;
        ho.index = d.d_ho_index;
        ho.id = d.d_ho_id;
        ho.flags = d.d_ho_flags;
        ho.deathtime_index = d.d_ho_dti;
        ho.capacity = (uint32_t)std::max<size_t>(pa_.n, 1);
        ho.evals = d.d_evals;
        ho.borderline = d.d_evals + 1;
        ho.learned = d.d_evals + 2;
        ho.wide = d.d_evals + 3;
        ck(cudaEventRecord(d.start, d.main), "event");
        int rc = launch_timeblock(&d.buf[d.cur].p, n_kernel, &pb, &sp, &ho, d.main);
        if (rc != GLISSER_OK) throw CudaError(std::string("time-block launch failed: ") + timeblock_error());
        ck(cudaEventRecord(d.stop, d.main), "event");
        launches_total_ += 1;
        // without encounter particles to bring back the partition follows the
        // kernel directly; otherwise after SWIFT's results are in place
        if (n_enc == 0) launch_partition_now();
    }
    // host work overlapped with the kernel
    auto c0 = clk::now();
    if (n_enc > 0) {
        auto ce = clk::now();
        handle_encounters(false, tm);
        tm.enc = ms_since(ce);
    } else {
        auto cp = clk::now();
        snapshot_ = pl_;
        t += cur_dt_ * (double)cur_tbsize_;
        update_planets();
        tm.planet = ms_since(cp);
    }
    double cpu = ms_since(c0);
    if (n_range > 0) {
        auto cr = clk::now();
        if (!partitioned) launch_partition_now();
        ck(cudaEventSynchronize(d.done), "block");
        if (n_kernel > 0) ck(cudaEventElapsedTime(&gpu, d.start, d.stop), "elapsed");
        uint32_t status = d.h_ctr[1];
        if (status) throw CudaError("time-block kernel reported a planet-log staging timeout");
        uint32_t n0 = d.h_ctr[2], n1 = d.h_ctr[3];
        uint32_t k = std::min<uint32_t>(d.h_ctr[0], (uint32_t)std::max<size_t>(pa_.n, 1));
        evals_total_ += d.h_evals[0];
        borderline_total_ += d.h_evals[1];
        learned_total_ += d.h_evals[2];
        wide_total_ += d.h_evals[3];
        if (n_kernel > 0) net_next_ = d.h_evals[3] > 0;
        // both particle buffers must agree on the particles that left the
        // partitioned range this block (the next partition reads only one)
        if (n0 + n1 < n_range) {
            int rc = launch_copy_range(&d.buf[d.cur].p, &d.buf[d.cur ^ 1].p, n0 + n1, n_range, d.main);
            if (rc != GLISSER_OK) throw CudaError("copy launch failed");
            launches_total_ += 1;
        }
        // particles that kept their flags advanced the whole block; the
        // flagged ones add their deathtime index below
        psteps_total_ += (unsigned long long)(n_kernel - std::min<size_t>(n_kernel, d.h_ctr[0])) * d.blk_len[used];
        n_dev_ = resolve ? n0 : n0 + n1;
        n_encounter_ = resolve ? n1 : 0;
        flagged_.clear();
        if (k) {
            auto cd = clk::now();
            ck(cudaMemcpyAsync(d.h_ho_id, d.d_ho_id, k * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.main), "hand-off");
            ck(cudaMemcpyAsync(d.h_ho_dti, d.d_ho_dti, k * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.main), "hand-off");
            ck(cudaMemcpyAsync(d.h_ho_flags, d.d_ho_flags, k * sizeof(uint16_t), cudaMemcpyDeviceToHost, d.main),
               "hand-off");
            ck(cudaStreamSynchronize(d.main), "hand-off sync");
            tm.dl = ms_since(cd);
            for (uint32_t q = 0; q < k; q++) {
                flagged_.push_back({ d.h_ho_id[q], d.h_ho_flags[q], d.h_ho_dti[q] });
                psteps_total_ += d.h_ho_dti[q];
            }
        }
        // particles SWIFT removed this block leave the alive range with them
        // (src/executor.cu:802-825 visits the whole range that left)
        for (size_t q = 0; q < n_enc; q++)
            if (enc_.flags[q] != 0) flagged_.push_back({ enc_.id[q], enc_.flags[q], enc_.dti[q] });
        // particles that entered the first block already in an encounter kept
        // their flag (the kernel reports only flags it changed)
        for (const FlaggedEntry& f : initial_flagged_) flagged_.push_back(f);
        initial_flagged_.clear();
        std::sort(flagged_.begin(), flagged_.end(),
                  [](const FlaggedEntry& a, const FlaggedEntry& b) { return a.id < b.id; });
        float tf = (float)t;
        for (auto& f : flagged_) {
            set_deathtime(f.id, tf);
            if ((f.flags & 0x04) && log)
                *log << "warning - particle " << f.id << " did not converge on GPU" << std::endl;
            if (encounter_out) {
                *encounter_out << std::setprecision(17) << f.id << ((f.flags & 0x80) ? " death " : " encounter ") << t
                               << "\n";
            }
        }
        // at the end of a lookup interval the particles that entered an
        // encounter in this block are brought to its end on SWIFT now, with
        // the interval that closed (src/executor.cu:837-873)
        if (resolve && starting_interval_ && n_encounter_ > 0) {
            auto ce = clk::now();
            handle_encounters(true, tm);
            tm.enc2 = ms_since(ce);
        }
        tm.resync = ms_since(cr);
    }
    tm.cpu = cpu;
    tm.gpu = gpu;
    tm.total = ms_since(t_total);
    timing_ = tm;
    if (timing_out) write_timing_row(tm, n_enc_start);
    if (cpu_ms) *cpu_ms = cpu;
    if (gpu_ms) *gpu_ms = gpu;
    return starting_interval_ || !cfg.resolve_encounters;
}

void Executor::EncounterSet::resize(size_t n)
{
    for (auto* a : { &rx, &ry, &rz, &vx, &vy, &vz, &ax, &ay, &az }) a->assign(n, 0.0);
    id.assign(n, 0);
    dti.assign(n, 0);
    flags.assign(n, 0);
}

void Executor::fetch_encounters(int buf, size_t begin, size_t n)
{
    Impl& d = *d_;
    enc_.resize(n);
    if (n == 0) return;
    const glisser_particles& p = d.buf[buf].p;
    const double* src[6] = { p.rx, p.ry, p.rz, p.vx, p.vy, p.vz };
    double* dst[6] = { enc_.rx.data(), enc_.ry.data(), enc_.rz.data(), enc_.vx.data(), enc_.vy.data(), enc_.vz.data() };
    // the side stream reads the encounter range while the kernel may still
    // be integrating the range before it
    for (int c = 0; c < 6; c++)
        ck(cudaMemcpyAsync(dst[c], src[c] + begin, n * sizeof(double), cudaMemcpyDeviceToHost, d.dth), "fetch");
    ck(cudaMemcpyAsync(enc_.id.data(), p.id + begin, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, d.dth), "fetch");
    ck(cudaMemcpyAsync(enc_.flags.data(), p.flags + begin, n * sizeof(uint16_t), cudaMemcpyDeviceToHost, d.dth),
       "fetch");
    ck(cudaStreamSynchronize(d.dth), "fetch sync");
}

void Executor::store_encounters(int buf, size_t begin, size_t n)
{
    Impl& d = *d_;
    if (n == 0) return;
    const glisser_particles& p = d.buf[buf].p;
    double* dst[9] = { p.rx, p.ry, p.rz, p.vx, p.vy, p.vz, p.ax, p.ay, p.az };
    const double* src[9] = { enc_.rx.data(), enc_.ry.data(), enc_.rz.data(), enc_.vx.data(), enc_.vy.data(),
                             enc_.vz.data(), enc_.ax.data(), enc_.ay.data(), enc_.az.data() };
    for (int c = 0; c < 9; c++)
        ck(cudaMemcpyAsync(dst[c] + begin, src[c], n * sizeof(double), cudaMemcpyHostToDevice, d.main), "store");
    ck(cudaMemcpyAsync(p.id + begin, enc_.id.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, d.main), "store");
    ck(cudaMemcpyAsync(p.flags + begin, enc_.flags.data(), n * sizeof(uint16_t), cudaMemcpyHostToDevice, d.main),
       "store");
    ck(cudaMemcpyAsync(p.deathtime_index + begin, enc_.dti.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice,
                       d.main),
       "store");
}

void Executor::encounter_accelerations(size_t n)
{
    // helio_acc_particle (src/wh.cpp:611-657) at the last step of the block
    // just integrated: h0 and the planet positions of that step (the old
    // log's last record) with the live masses and encounter radii.  Its
    // flags overwrite SWIFT's; a close-encounter flag is then cleared so that
    // the next block detects the encounter itself (src/executor.cu:566-576).
    const Planets& P = snapshot_;
    const size_t npl_old = P.n_alive;
    std::vector<double> pos(3 * (npl_old > 0 ? npl_old - 1 : 0));
    for (size_t j = 1; j < npl_old; j++) {
        pos[3 * (j - 1)] = P.r[j].x;
        pos[3 * (j - 1) + 1] = P.r[j].y;
        pos[3 * (j - 1) + 2] = P.r[j].z;
    }
    const Vec3 h0 = npl_old > 1 ? indirect_term(pos.data(), P.m, npl_old) : Vec3{ 0, 0, 0 };
    const size_t npl = std::min(pl_.n_alive, npl_old);
    const double outer2 = cfg.outer_radius * cfg.outer_radius;
    const float tf = (float)t;
    for (size_t k = 0; k < n; k++) {
        const Vec3 r{ enc_.rx[k], enc_.ry[k], enc_.rz[k] };
        Vec3 a = h0;
        uint16_t fl = enc_.flags[k];
        bool stamped = false;
        for (size_t j = 1; j < npl; j++) {
            Vec3 dr = r - P.r[j];
            double r2 = dr.lensq();
            double inv3 = 1. / (r2 * std::sqrt(r2));
            double fac = pl_.m[j] * inv3;
            a -= dr * fac;
            if (r2 < rh_[j] * rh_[j]) {
                stamped = true;
                fl = (uint16_t)((j << 8) | 0x0001);
            }
        }
        double r2 = r.lensq();
        if (r2 < rh_[0] * rh_[0]) {
            stamped = true;
            fl = 0x0001;
        }
        if (r2 > outer2) {
            stamped = true;
            fl = 0x0002;
        }
        if (stamped) set_deathtime(enc_.id[k], tf);
        if ((fl & 0xFF) == 0x01) fl = 0;
        enc_.flags[k] = fl;
        enc_.ax[k] = a.x;
        enc_.ay[k] = a.y;
        enc_.az[k] = a.z;
        // the host's deathtime index travels back with the state; the
        // reference never downloads it, so it is the zero it started with
        enc_.dti[k] = 0;
    }
}

void Executor::handle_encounters(bool from_resync, BlockTiming& tm)
{
    // Executor::handle_encounters (src/executor.cu:470-596).  Called in
    // step_block while the kernel integrates the current block (SWIFT
    // resumes the encounter particles from the start of the previous block
    // to the end of the current one), or after the partition at the end of
    // a lookup interval (from the start of the block just integrated to the
    // interval's end).
    Impl& d = *d_;
    auto& ip = interp_;
    const size_t begin = n_dev_;
    const size_t n = n_encounter_;
    const size_t prev_len = (starting_interval_ && !from_resync) ? 0 : prev_tbsize_;
    const size_t cur_len = from_resync ? 0 : cur_tbsize_;
    const double which_dt = from_resync ? prev_dt_ : cur_dt_;
    if (from_resync && !(std::abs(ip.t0 - t) < 1e-2))
        throw std::runtime_error("sanity check failed: end-of-chunk encounter time");
    const double rel_t = from_resync ? ip.t0 - ip.t_m1 : ip.rel_t - ip.eff_dt * (double)cur_tbsize_;
    const auto clocks = clk::now();
    fetch_encounters(d.cur, begin, n);
    std::vector<Vec3> r(n), v(n);
    for (size_t k = 0; k < n; k++) {
        r[k] = Vec3{ enc_.rx[k], enc_.ry[k], enc_.rz[k] };
        v[k] = Vec3{ enc_.vx[k], enc_.vy[k], enc_.vz[k] };
    }
    // the lookup interval SWIFT integrates in: the current one, or at an
    // interval boundary the one that just closed
    SwiftHistory h;
    h.m0 = pl_.m[0];
    const std::vector<uint32_t>* planet_ids;
    if (from_resync) {
        const auto& o = ip.old;
        h.span = ip.t0 - ip.t_m1;
        h.npl = o.n_alive;
        h.ids = o.ids.data(); h.mass = o.mass.data();
        h.aei_i = o.aei_i.data(); h.oom_i = o.oom_i.data(); h.aei_f = o.aei_f.data(); h.oom_f = o.oom_f.data();
        planet_ids = &o.ids;
    } else {
        h.span = ip.t1 - ip.t0;
        h.npl = ip.n_alive;
        h.ids = ip.ids.data(); h.mass = ip.mass.data();
        h.aei_i = ip.aei_i.data(); h.oom_i = ip.oom_i.data(); h.aei_f = ip.aei_f.data(); h.oom_f = ip.oom_f.data();
        planet_ids = &ip.ids;
    }
    double wswift = 0, iswift = 0, rswift = 0, dswift = 0;
    swift_->begin(h, *planet_ids, n, r.data(), v.data(), rel_t, which_dt, prev_len, cur_len, &wswift, &iswift);
    if (!from_resync) {
        // the planets of the next block while SWIFT runs (outputs are written
        // by the caller after step_block returns)
        auto cp = clk::now();
        try {
            snapshot_ = pl_;
            t += cur_dt_ * (double)cur_tbsize_;
            update_planets();
        } catch (...) {
            swift_->reap();
            throw;
        }
        tm.planet = ms_since(cp);
    }
    swift_->end(n, enc_.id.data(), r.data(), v.data(), enc_.flags.data(), &rswift, &dswift);
    if (!from_resync) {
        tm.wswift = wswift;
        tm.iswift = iswift;
        tm.rswift = rswift;
        tm.dswift = dswift;
        tm.swift = ms_since(clocks);
    }
    for (size_t k = 0; k < n; k++) {
        if (!std::isfinite(r[k].x) || !std::isfinite(r[k].y) || !std::isfinite(r[k].z) || !std::isfinite(v[k].x) ||
            !std::isfinite(v[k].y) || !std::isfinite(v[k].z))
            throw std::runtime_error("SWIFT returned a non-finite state for particle " + std::to_string(enc_.id[k]));
        enc_.rx[k] = r[k].x; enc_.ry[k] = r[k].y; enc_.rz[k] = r[k].z;
        enc_.vx[k] = v[k].x; enc_.vy[k] = v[k].y; enc_.vz[k] = v[k].z;
    }
    encounter_accelerations(n);
    auto cu = clk::now();
    if (!from_resync) {
        // into the range after the unflagged particles of the running
        // kernel's buffer; the partition after the block sorts them in
        store_encounters(d.cur, begin, n);
    } else {
        // sort the range here: unflagged, encounter, removed (the partial
        // partitions of src/executor.cu:849-858); what follows it is removed
        std::vector<size_t> order(n);
        std::iota(order.begin(), order.end(), 0);
        auto m1 = std::stable_partition(order.begin(), order.end(), [&](size_t q) { return enc_.flags[q] == 0; });
        auto m2 = std::stable_partition(m1, order.end(), [&](size_t q) { return (enc_.flags[q] & 0xFE) == 0; });
        const size_t n_ok = (size_t)(m1 - order.begin()), n_e = (size_t)(m2 - m1);
        EncounterSet s = enc_;
        for (size_t q = 0; q < n; q++) {
            size_t o = order[q];
            enc_.rx[q] = s.rx[o]; enc_.ry[q] = s.ry[o]; enc_.rz[q] = s.rz[o];
            enc_.vx[q] = s.vx[o]; enc_.vy[q] = s.vy[o]; enc_.vz[q] = s.vz[o];
            enc_.ax[q] = s.ax[o]; enc_.ay[q] = s.ay[o]; enc_.az[q] = s.az[o];
            enc_.id[q] = s.id[o]; enc_.dti[q] = s.dti[o]; enc_.flags[q] = s.flags[o];
        }
        // both buffers: the removed ones lie outside the next partition's range
        store_encounters(d.cur, begin, n);
        store_encounters(d.cur ^ 1, begin, n);
        n_dev_ = begin + n_ok;
        n_encounter_ = n_e;
        host_dirty_ = true;
    }
    ck(cudaStreamSynchronize(d.main), "store sync");
    tm.encup = ms_since(cu);
}

void Executor::write_timing_header()
{
    *timing_out << "t,      n_enc,  enc,    wswift, iswift, swift,  rswift, dswift, io,     planet, planetu,encup,  "
                   "sort,   dl,     endenc, resync, cpu,    gpu,    total"
                << std::endl;
}

void Executor::write_timing_row(const BlockTiming& tm, size_t n_enc)
{
    std::ostream& o = *timing_out;
    o << std::left << std::fixed << std::setprecision(3);
    const double cols[19] = { t, (double)n_enc, tm.enc, tm.wswift, tm.iswift, tm.swift, tm.rswift,
                              tm.dswift, tm.io, tm.planet, tm.planetu, tm.encup, tm.sort, tm.dl, tm.enc2,
                              tm.resync, tm.cpu, tm.gpu, tm.total };
    for (int c = 0; c < 19; c++) {
        if (c == 1) o << std::setw(8) << (size_t)cols[c];
        else o << std::setw(8) << cols[c];
    }
    o << std::endl;
}

void Executor::finish()
{
    // stat.out: SWIFT's status of every particle handed to it
    // (src/executor.cu:880-882; empty when none was)
    if (!cfg.outfolder.empty()) {
        std::ofstream st(cfg.outfolder + "/stat.out");
        if (swift_) swift_->stats.write(st);
    }
    if (initialized_ && d_->device) {
        ck(cudaStreamSynchronize(d_->main), "finish");
        download_particles();
    }
    if (log) *log << "Simulation finished. t = " << t << ". n_particle = " << n_alive_host() << std::endl;
}

}  // namespace glisser
