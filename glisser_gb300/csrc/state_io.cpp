// State, track and history file formats.
//
// Text layouts and number formatting (17 significant digits, one record per
// line) and the binary field order are the reference's (src/data.cpp), so
// files written here load in the reference's tools and vice versa.  Two
// deliberate differences, both documented:
//  * the binary reader reads the particle deathtime as f64, the type the
//    reference's own writer emits (the reference reader takes f32 and so
//    misreads its own binary dumps);
//  * readers check for truncation and throw instead of leaving zeros.
#include "state_io.h"
#include "parallel.h"

#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <limits>
#include <sstream>
#include <sys/stat.h>

namespace glisser {

namespace {

template <typename T>
void put(std::ostream& o, T x)
{
    o.write(reinterpret_cast<const char*>(&x), sizeof(T));
}

template <typename T>
T get(std::istream& in)
{
    T x{};
    in.read(reinterpret_cast<char*>(&x), sizeof(T));
    return x;
}

bool file_exists(const std::string& p)
{
    struct stat s;
    return stat(p.c_str(), &s) == 0 && S_ISREG(s.st_mode);
}

std::istringstream line_stream(std::istream& in)
{
    std::string s;
    std::getline(in, s);
    return std::istringstream(s);
}

void load_hybrid_ascii(std::istream& in, const Config& cfg, Planets& pl, Particles& pa)
{
    size_t npl = 0;
    line_stream(in) >> npl;
    pl.resize(npl);
    pl.n_alive = npl;
    for (size_t i = 0; i < npl; i++) {
        line_stream(in) >> pl.m[i];
        { auto ss = line_stream(in); ss >> pl.r[i].x >> pl.r[i].y >> pl.r[i].z; }
        { auto ss = line_stream(in); ss >> pl.v[i].x >> pl.v[i].y >> pl.v[i].z; }
        line_stream(in) >> pl.id[i];
    }
    size_t npart = 0;
    line_stream(in) >> npart;
    npart = std::min(npart, (size_t)cfg.max_particle);
    pa.resize(npart);
    for (size_t i = 0; i < npart; i++) {
        { auto ss = line_stream(in); ss >> pa.r[i].x >> pa.r[i].y >> pa.r[i].z; }
        { auto ss = line_stream(in); ss >> pa.v[i].x >> pa.v[i].y >> pa.v[i].z; }
        auto ss = line_stream(in);
        ss >> pa.id[i] >> pa.flags[i];
        ss >> pa.deathtime[i];
    }
    if (in.bad()) throw IoError("could not read the input state");
}

void load_hybrid_binary(std::istream& in, const Config& cfg, Planets& pl, Particles& pa)
{
    size_t npl = (size_t)get<uint64_t>(in);
    if (!in || npl > 1u << 20) throw IoError("binary state: bad planet count");
    pl.resize(npl);
    pl.n_alive = npl;
    for (size_t i = 0; i < npl; i++) {
        pl.id[i] = get<uint32_t>(in);
        pl.m[i] = get<double>(in);
        pl.r[i] = Vec3{ get<double>(in), get<double>(in), get<double>(in) };
        pl.v[i] = Vec3{ get<double>(in), get<double>(in), get<double>(in) };
    }
    size_t npart = std::min((size_t)get<uint64_t>(in), (size_t)cfg.max_particle);
    if (!in) throw IoError("binary state: truncated");
    pa.resize(npart);
    for (size_t i = 0; i < npart; i++) {
        pa.id[i] = get<uint32_t>(in);
        pa.r[i] = Vec3{ get<double>(in), get<double>(in), get<double>(in) };
        pa.v[i] = Vec3{ get<double>(in), get<double>(in), get<double>(in) };
        pa.flags[i] = get<uint16_t>(in);
        pa.deathtime[i] = get<double>(in);
    }
    if (!in) throw IoError("binary state: truncated");
}

// src/data.cpp:374-425 (planet file: count, then m x y z vx vy vz per planet;
// particle file: count, then x y z vx vy vz [deathtime flags id] per particle)
void load_split(std::istream& plin, std::istream& icsin, const Config& cfg, Planets& pl, Particles& pa)
{
    size_t npl = 0;
    plin >> npl;
    pl.resize(npl);
    pl.n_alive = npl;
    for (size_t i = 0; i < npl; i++) {
        plin >> pl.m[i] >> pl.r[i].x >> pl.r[i].y >> pl.r[i].z >> pl.v[i].x >> pl.v[i].y >> pl.v[i].z;
        pl.id[i] = (uint32_t)i;
    }
    size_t npart = 0;
    icsin >> npart;
    npart = std::min(npart, (size_t)cfg.max_particle);
    pa.resize(npart);
    for (size_t i = 0; i < npart; i++) {
        icsin >> pa.r[i].x >> pa.r[i].y >> pa.r[i].z >> pa.v[i].x >> pa.v[i].y >> pa.v[i].z;
        std::string s;
        icsin >> s;
        if (s.empty() || !std::isdigit((unsigned char)s[0])) {
            icsin.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
            pa.deathtime[i] = 0;
            pa.id[i] = (uint32_t)i;
            pa.flags[i] = 0;
        } else {
            pa.deathtime[i] = std::stof(s);
            icsin >> pa.flags[i] >> pa.id[i];
        }
    }
}

}  // namespace

void load_state(const Config& cfg, Planets& pl, Particles& pa)
{
    if (cfg.readsplit) {
        if (!file_exists(cfg.plin)) throw IoError("Planet input file " + cfg.plin + " does not exist");
        if (!file_exists(cfg.icsin)) throw IoError("Particle input file " + cfg.icsin + " does not exist");
        std::ifstream p(cfg.plin), c(cfg.icsin);
        load_split(p, c, cfg, pl, pa);
    } else {
        if (!file_exists(cfg.hybridin)) throw IoError("Input file " + cfg.hybridin + " does not exist");
        if (cfg.readbinary) {
            std::ifstream in(cfg.hybridin, std::ios::binary);
            load_hybrid_binary(in, cfg, pl, pa);
        } else {
            std::ifstream in(cfg.hybridin);
            load_hybrid_ascii(in, cfg, pl, pa);
        }
    }
    for (size_t i = 0; i < pl.n; i++) {
        if (cfg.readmomenta) pl.v[i] = pl.v[i] / pl.m[i];
        pl.m[i] *= cfg.big_g;
    }
}

void save_state_ascii(std::ostream& out, const Config& cfg, const Planets& pl, const Particles& pa)
{
    out << pl.n_alive << std::endl;
    out << std::setprecision(17);
    for (size_t i = 0; i < pl.n_alive; i++) {
        double m = pl.m[i];
        out << m << std::endl;
        if (!cfg.writemomenta) m = 1;
        out << pl.r[i].x << " " << pl.r[i].y << " " << pl.r[i].z << std::endl;
        out << pl.v[i].x * m << " " << pl.v[i].y * m << " " << pl.v[i].z * m << std::endl;
        out << pl.id[i] << std::endl;
    }
    out << pa.n << std::endl;
    for (size_t i = 0; i < pa.n; i++) {
        out << pa.r[i].x << " " << pa.r[i].y << " " << pa.r[i].z << std::endl;
        out << pa.v[i].x << " " << pa.v[i].y << " " << pa.v[i].z << std::endl;
        out << pa.id[i] << " " << pa.flags[i] << " " << pa.deathtime[i] << std::endl;
    }
}

void save_state_binary(std::ostream& out, const Config& cfg, const Planets& pl, const Particles& pa)
{
    put<uint64_t>(out, pl.n_alive);
    for (size_t i = 0; i < pl.n_alive; i++) {
        double m = pl.m[i];
        put<uint32_t>(out, pl.id[i]);
        put<double>(out, m);
        if (!cfg.writemomenta) m = 1;
        put(out, pl.r[i].x); put(out, pl.r[i].y); put(out, pl.r[i].z);
        put(out, pl.v[i].x * m); put(out, pl.v[i].y * m); put(out, pl.v[i].z * m);
    }
    put<uint64_t>(out, pa.n);
    // packed 62-byte records (id, r, v, flags, deathtime) formatted in memory
    // across the host cores, then one write
    constexpr size_t REC = 4 + 6 * 8 + 2 + 8;
    std::vector<char> buf(pa.n * REC);
    parallel_for(pa.n, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; i++) {
            char* q = buf.data() + i * REC;
            const double rv[6] = { pa.r[i].x, pa.r[i].y, pa.r[i].z, pa.v[i].x, pa.v[i].y, pa.v[i].z };
            std::memcpy(q, &pa.id[i], 4);
            std::memcpy(q + 4, rv, 48);
            std::memcpy(q + 52, &pa.flags[i], 2);
            std::memcpy(q + 54, &pa.deathtime[i], 8);
        }
    });
    out.write(buf.data(), (std::streamsize)buf.size());
}

void save_state(const Config& cfg, const Planets& pl, const Particles& pa, const std::string& path)
{
    if (!cfg.writesplit) {
        std::ofstream out(path, cfg.writebinary ? std::ios::binary : std::ios::out);
        if (!out) throw IoError("cannot write " + path);
        if (cfg.writebinary) save_state_binary(out, cfg, pl, pa);
        else save_state_ascii(out, cfg, pl, pa);
        return;
    }
    // split output (src/data.cpp:645-668): pl.out and ics.out in Output-Folder
    std::ofstream plo(cfg.outfolder + "/pl.out"), ics(cfg.outfolder + "/ics.out");
    plo << pl.n_alive << std::endl << std::setprecision(17);
    for (size_t i = 0; i < pl.n_alive; i++) {
        double m = pl.m[i];
        plo << m << std::endl;
        if (!cfg.writemomenta) m = 1;
        plo << pl.r[i].x << " " << pl.r[i].y << " " << pl.r[i].z << std::endl;
        plo << pl.v[i].x * m << " " << pl.v[i].y * m << " " << pl.v[i].z * m << std::endl;
    }
    ics << pa.n << std::endl << std::setprecision(17);
    for (size_t i = 0; i < pa.n; i++) {
        ics << pa.r[i].x << " " << pa.r[i].y << " " << pa.r[i].z << std::endl;
        ics << pa.v[i].x << " " << pa.v[i].y << " " << pa.v[i].z << std::endl;
        ics << pa.deathtime[i] << " " << pa.flags[i] << " " << pa.id[i] << std::endl;
    }
}

void write_track_planets(std::ostream& out, const Planets& pl, double time, bool barycentric)
{
    put<double>(out, time);
    put<uint64_t>(out, pl.n_alive > 0 ? pl.n_alive - 1 : 0);
    for (size_t i = 1; i < pl.n_alive; i++) {
        double cm = pl.m[0];
        Vec3 cr = pl.r[0] * pl.m[0], cv = pl.v[0] * pl.m[0];
        if (barycentric) {
            for (size_t j = 1; j < pl.n_alive; j++) {
                if (j == i) continue;
                cm += pl.m[j];
                cr += pl.r[j] * pl.m[j];
                cv += pl.v[j] * pl.m[j];
            }
        }
        cr = cr / cm;
        cv = cv / cm;
        Elements el = to_elements(pl.m[i] + cm, pl.r[i] - cr, pl.v[i] - cv);
        put<uint32_t>(out, pl.id[i]);
        put<float>(out, (float)el.a); put<float>(out, (float)el.e); put<float>(out, (float)el.i);
        put<float>(out, (float)el.capom); put<float>(out, (float)el.om); put<float>(out, (float)el.f);
    }
}

void track_particle_frame(const Planets& pl, bool barycentric, double& cm, Vec3& cr, Vec3& cv)
{
    cm = pl.m[0];
    cr = pl.r[0];
    cv = pl.v[0];
    if (barycentric) {
        Vec3 rs{ 0, 0, 0 }, vs{ 0, 0, 0 };
        cm = 0;
        for (size_t j = 0; j < pl.n_alive; j++) {
            rs += pl.r[j] * pl.m[j];
            vs += pl.v[j] * pl.m[j];
            cm += pl.m[j];
        }
        cr = rs / cm;
        cv = vs / cm;
    }
}

void write_track(std::ostream& out, const Planets& pl, const Particles& pa, const std::vector<size_t>& order,
                 double time, bool barycentric)
{
    write_track_planets(out, pl, time, barycentric);
    put<uint64_t>(out, order.size());
    double cm;
    Vec3 cr, cv;
    track_particle_frame(pl, barycentric, cm, cr, cv);
    for (size_t k : order) {
        Elements el = to_elements(cm, pa.r[k] - cr, pa.v[k] - cv);
        put<uint32_t>(out, pa.id[k]);
        put<float>(out, (float)el.a); put<float>(out, (float)el.e); put<float>(out, (float)el.i);
        put<float>(out, (float)el.capom); put<float>(out, (float)el.om); put<float>(out, (float)el.f);
    }
    out.flush();
}

void write_plhist_header(std::ostream& out, const Planets& pl)
{
    put<double>(out, pl.m[0]);
    for (int k = 0; k < 24; k++) put<uint8_t>(out, 0);
}

void write_plhist_record(std::ostream& out, const Planets& pl, double time)
{
    put<double>(out, time);
    put<uint32_t>(out, pl.n_alive > 0 ? (uint32_t)(pl.n_alive - 1) : 0u);
    for (int k = 0; k < 20; k++) put<uint8_t>(out, 0);
    for (size_t i = 1; i < pl.n_alive; i++) {
        // heliocentric elements (the history is always heliocentric)
        double cm = pl.m[0];
        Vec3 cr = pl.r[0] * pl.m[0] / cm, cv = pl.v[0] * pl.m[0] / cm;
        Elements el = to_elements(pl.m[i] + cm, pl.r[i] - cr, pl.v[i] - cv);
        put<uint32_t>(out, pl.id[i]);
        put<float>(out, (float)pl.m[i]);
        put<float>(out, (float)el.a); put<float>(out, (float)el.e); put<float>(out, (float)el.i);
        put<float>(out, (float)el.capom); put<float>(out, (float)el.om);
        put<float>(out, (float)mean_anomaly(el.e, el.f));
    }
    out.flush();
}

}  // namespace glisser
