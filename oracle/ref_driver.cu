// Test infrastructure only: a C-ABI driver around the UNMODIFIED reference
// sources, compiled from where they lie by oracle/build_ref.sh into
// oracle/_ref/libglisser_ref.so.  It is used in this container to pin the
// oracle restatement (oracle/glisser_oracle.c) and to generate the golden
// fixtures under tests/golden/.  Nothing in the product links it.
//
// The particle kernel arithmetic is the reference's own
// MVSKernel::step_forward (src/wh.cu:113-177), which is __host__ __device__:
// including src/wh.cu in this host translation unit runs exactly that code on
// the CPU.  The block loop below restates Executor::init / update_planets /
// loop / resync2 / handle_encounters (src/executor.cu:85-217, 226-320,
// 470-596, 598-764, 766-877) on top of the reference's WHIntegrator
// (src/wh.cpp), Interpolator (src/interp.cpp) and, with Resolve-Encounters,
// SwiftEncounterIntegrator (src/swift.cpp), which runs Swift-Path itself.
// One set of particle arrays stands for both the device arrays and the host
// mirror; where the two differ in the reference (the rollback state the host
// reads back, the host's never-downloaded deathtime index) the emulation
// says so.

#include "wh.cu"
#include "interp.h"
#include "convert.h"
#include "data.h"
#include "swift.h"

#include <algorithm>
#include <iomanip>
#include <cstring>
#include <fstream>
#include <numeric>
#include <sstream>
#include <string>

using namespace sr::data;

namespace
{
	struct RefExec
	{
		Configuration config;
		HostData hd;
		sr::wh::WHIntegrator integ;
		sr::interp::Interpolator interp;

		double t = 0;
		double cur_dt = 0, prev_dt = 0;
		size_t cur_tbsize = 0, prev_tbsize = 0;
		bool starting_lookup_interval = false;

		// "device" copies of the planet block, as upload_planet_log would leave them
		Vf64_3 dev_r_log, dev_h0_log;
		Vf64 dev_m, dev_rh;
		Vu32 dev_id;
		uint32_t dev_npl = 0, dev_len = 0;

		// particle acceleration in device order
		Vf64_3 dev_a;
		size_t dev_n_alive = 0;
		std::string err;
		std::ostringstream log;

		// Resolve-Encounters: the encounter integrator, the rollback state
		// (r, v in device order), the presort boundary, and a record of every
		// hand-off for the tests
		sr::swift::SwiftEncounterIntegrator swift;
		Vf64_3 rb_r, rb_v;
		size_t presort = 0;
		struct SwiftCall
		{
			int old;
			double t, rel_t, dt;
			size_t prev_len, cur_len, begin, n;
			Vu32 ids;
			Vf64_3 r_in, v_in, r_out, v_out;
			Vu16 flags_out;
		};
		std::vector<SwiftCall> calls;
	};

	void upload_planets(RefExec& e)
	{
		e.dev_r_log = e.hd.planets.r_log().log;
		e.dev_m = e.hd.planets.m();
		e.dev_id = e.hd.planets.id();
		e.dev_npl = static_cast<uint32_t>(e.hd.planets.n_alive());
		e.dev_len = static_cast<uint32_t>(e.hd.planets.r_log().len);
		e.dev_rh = e.integ.planet_rh;
		e.dev_h0_log = e.integ.planet_h0_log.log;
	}

	void update_planets(RefExec& e)
	{
		e.prev_dt = e.cur_dt;
		e.prev_tbsize = e.cur_tbsize;
		e.integ.recalculate_rh(e.hd.planets);
		auto& ip = e.interp;
		if (e.config.interp_planets)
		{
			if (ip.cur_ts == ip.n_ts)
			{
				ip.next(e.hd.planets);
				ip.cur_ts = 0;
				e.t = ip.t0;
				e.starting_lookup_interval = true;
			}
			else
			{
				e.starting_lookup_interval = ip.cur_ts == 0;
			}
			e.cur_dt = ip.eff_dt;
			e.cur_tbsize = std::min(e.config.tbsize, static_cast<uint32_t>(ip.n_ts - ip.cur_ts));
			ip.fill(e.hd.planets, e.cur_tbsize, ip.rel_t, e.cur_dt);
			ip.rel_t += static_cast<double>(e.cur_tbsize) * e.cur_dt;
			ip.cur_ts += e.cur_tbsize;
			e.integ.load_h0(e.hd.planets);
		}
		else
		{
			e.cur_dt = e.config.dt;
			e.cur_tbsize = e.config.tbsize;
			e.integ.integrate_planets_timeblock(e.hd.planets, e.cur_tbsize, e.t, e.cur_dt);
		}
		e.hd.planets.swap_logs();
		e.integ.swap_logs();
		upload_planets(e);
	}

	// stable partition of [begin, end) by pred, moving every per-particle
	// array the reference's device partition moves
	template<typename P>
	size_t partition_all(RefExec& e, size_t begin, size_t end, P pred)
	{
		auto& pa = e.hd.particles;
		if (end <= begin) return begin;
		Vs idx(end - begin);
		std::iota(idx.begin(), idx.end(), 0);
		auto mid = std::stable_partition(idx.begin(), idx.end(), [&](size_t k) { return pred(pa.deathflags()[begin + k]); });
		size_t boundary = begin + static_cast<size_t>(mid - idx.begin());
		pa.gather(idx, begin, end - begin);
		gather(pa.deathtime_index(), idx, begin, end - begin);
		gather(e.dev_a, idx, begin, end - begin);
		gather(e.rb_r, idx, begin, end - begin);
		gather(e.rb_v, idx, begin, end - begin);
		return boundary;
	}

	bool unflagged(uint16_t f) { return f == 0; }
	bool alive(uint16_t f) { return (f & 0x00FE) == 0; }

	// Executor::handle_encounters (src/executor.cu:470-596)
	void handle_encounters(RefExec& e, bool called_from_resync)
	{
		auto& pa = e.hd.particles;
		auto& ip = e.interp;
		size_t encounter_start = pa.n_alive() - pa.n_encounter();
		size_t prev_len = e.prev_tbsize;
		if (e.starting_lookup_interval && !called_from_resync) prev_len = 0;
		size_t cur_len = called_from_resync ? 0 : e.cur_tbsize;
		double which_dt = called_from_resync ? e.prev_dt : e.cur_dt;
		if (called_from_resync && !(std::abs(ip.t0 - e.t) < 1e-2)) throw std::runtime_error("end-of-chunk encounter time");
		double rel_t = called_from_resync ? ip.t0 - ip.t_m1 : ip.rel_t - ip.eff_dt * static_cast<double>(e.cur_tbsize);
		double which_t = called_from_resync ? ip.t0 : ip.t0 + rel_t;

		RefExec::SwiftCall call;
		call.old = called_from_resync ? 1 : 0;
		call.t = which_t; call.rel_t = rel_t; call.dt = which_dt;
		call.prev_len = prev_len; call.cur_len = cur_len;
		call.begin = encounter_start; call.n = pa.n_encounter();
		for (size_t i = encounter_start; i < encounter_start + call.n; i++)
		{
			call.ids.push_back(pa.id()[i]);
			call.r_in.push_back(pa.r()[i]);
			call.v_in.push_back(pa.v()[i]);
		}

		e.swift.begin_integrate(e.hd.planets, pa, ip, called_from_resync, which_t, rel_t, which_dt, prev_len, cur_len);
		if (!called_from_resync)
		{
			e.hd.planets_snapshot = e.hd.planets.base;
			e.t += e.cur_dt * static_cast<double>(e.cur_tbsize);
			update_planets(e);
		}
		e.swift.end_integrate(pa);
		for (size_t i = encounter_start; i < encounter_start + call.n; i++)
		{
			call.r_out.push_back(pa.r()[i]);
			call.v_out.push_back(pa.v()[i]);
			call.flags_out.push_back(pa.deathflags()[i]);
		}
		e.calls.push_back(call);

		e.integ.helio_acc_particles(e.hd.planets, pa, encounter_start, pa.n_encounter(), e.t,
			e.hd.planets.r_log().len_old - 1, true);
		for (size_t i = encounter_start; i < encounter_start + pa.n_encounter(); i++)
		{
			if ((pa.deathflags()[i] & 0xFF) == 0x01) pa.deathflags()[i] = 0;
			// upload_data: the host's deathtime index, never downloaded, is zero
			pa.deathtime_index()[i] = 0;
			e.dev_a[i] = e.integ.particle_a[i];
		}
		e.dev_n_alive = pa.n_alive();
	}

	// Executor::resync2 (src/executor.cu:766-877) with Resolve-Encounters
	void resync_resolve(RefExec& e)
	{
		auto& pa = e.hd.particles;
		size_t prev_alive = e.dev_n_alive;
		e.dev_n_alive = partition_all(e, e.presort, prev_alive, unflagged);
		pa.n_encounter() = partition_all(e, e.dev_n_alive, prev_alive, alive) - e.dev_n_alive;
		pa.n_alive() = e.dev_n_alive + pa.n_encounter();
		for (size_t i = e.dev_n_alive; i < prev_alive; i++)
		{
			pa.deathtime_map()[pa.id()[i]] = static_cast<float>(e.t);
			e.log << pa.id()[i] << ((pa.deathflags()[i] & 0x80) ? " death " : " encounter ") << e.t << "\n";
		}
		// the host reads the encounter particles' rollback state
		for (size_t i = e.dev_n_alive; i < e.dev_n_alive + pa.n_encounter(); i++)
		{
			pa.r()[i] = e.rb_r[i];
			pa.v()[i] = e.rb_v[i];
		}
		if (e.starting_lookup_interval && pa.n_encounter() > 0)
		{
			size_t n_encounters = pa.n_encounter();
			handle_encounters(e, true);
			e.dev_n_alive = partition_all(e, e.dev_n_alive - n_encounters, e.dev_n_alive, unflagged);
			pa.n_encounter() = partition_all(e, e.dev_n_alive, prev_alive, alive) - e.dev_n_alive;
			pa.n_alive() = e.dev_n_alive + pa.n_encounter();
		}
	}

	// Executor::loop (src/executor.cu:598-764) with Resolve-Encounters
	void loop_resolve(RefExec& e)
	{
		auto& pa = e.hd.particles;
		if (e.dev_n_alive > 0)
		{
			e.rb_r = pa.r();
			e.rb_v = pa.v();
			for (size_t i = 0; i < e.dev_n_alive; i++)
			{
				uint32_t d = 0;
				sr::wh::MVSKernel::step_forward(pa.r()[i], pa.v()[i], pa.deathflags()[i], e.dev_a[i], d,
					e.dev_len, e.dev_npl, e.dev_h0_log.data(), e.dev_r_log.data(), e.dev_m.data(),
					e.dev_id.data(), e.dev_rh.data(), e.config.outer_radius, e.cur_dt, e.dev_m[0]);
				pa.deathtime_index()[i] = d;
			}
			e.presort = partition_all(e, 0, e.dev_n_alive, unflagged);
		}
		if (pa.n_encounter() > 0)
		{
			handle_encounters(e, false);
		}
		else
		{
			e.hd.planets_snapshot = e.hd.planets.base;
			e.t += e.cur_dt * static_cast<double>(e.cur_tbsize);
			update_planets(e);
		}
		if (e.dev_n_alive > 0) resync_resolve(e);
	}
}

extern "C"
{
	// One time block of the reference particle kernel on n particles.  Vectors
	// are [n][3] doubles; the planet log is [tbsize][planet_n-1][3].
	void ref_mvs_block(size_t n, double* r, double* v, double* a, uint16_t* flags, uint32_t* dti,
		uint32_t tbsize, uint32_t planet_n, const double* h0_log, const double* r_log,
		const double* m, const uint32_t* pl_id, const double* rh, double outer_r, double dt, double mu)
	{
		const f64_3* h0 = reinterpret_cast<const f64_3*>(h0_log);
		const f64_3* rl = reinterpret_cast<const f64_3*>(r_log);
		for (size_t i = 0; i < n; i++)
		{
			f64_3 ri(r[3 * i], r[3 * i + 1], r[3 * i + 2]);
			f64_3 vi(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
			f64_3 ai(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
			uint16_t fl = flags[i];
			uint32_t d = 0;
			sr::wh::MVSKernel::step_forward(ri, vi, fl, ai, d, tbsize, planet_n, h0, rl, m, pl_id, rh, outer_r, dt, mu);
			r[3 * i] = ri.x; r[3 * i + 1] = ri.y; r[3 * i + 2] = ri.z;
			v[3 * i] = vi.x; v[3 * i + 1] = vi.y; v[3 * i + 2] = vi.z;
			a[3 * i] = ai.x; a[3 * i + 1] = ai.y; a[3 * i + 2] = ai.z;
			flags[i] = fl;
			dti[i] = d;
		}
	}

	int ref_kepu(double dt, double r0, double mu, double alpha, double u, double* fp, double* c1, double* c2, double* c3)
	{
		return sr::wh::kepu(dt, r0, mu, alpha, u, fp, c1, c2, c3) ? 1 : 0;
	}

	void ref_from_elements_M(double mu, double a, double e, double i, double capom, double om, double M, double* r, double* v)
	{
		f64_3 rr, vv;
		sr::convert::from_elements_M(mu, a, e, i, capom, om, M, &rr, &vv);
		r[0] = rr.x; r[1] = rr.y; r[2] = rr.z;
		v[0] = vv.x; v[1] = vv.y; v[2] = vv.z;
	}

	void ref_to_elements(double mu, const double* r, const double* v, int* esign, double* out6)
	{
		sr::convert::to_elements(mu, f64_3(r[0], r[1], r[2]), f64_3(v[0], v[1], v[2]), esign,
			out6, out6 + 1, out6 + 2, out6 + 3, out6 + 4, out6 + 5);
	}

	double ref_mean_anomaly(double e, double f) { return sr::convert::get_mean_anomaly(e, f); }

	// ---- executor emulation -------------------------------------------------

	void* ref_exec_create(const char* config_text)
	{
		RefExec* e = new RefExec();
		try
		{
			std::istringstream in(config_text);
			read_configuration(in, &e->config);
			if (load_data(e->hd.planets, e->hd.particles, e->config))
			{
				delete e;
				return nullptr;
			}
			e->t = e->config.t_0;
		}
		catch (std::exception& ex)
		{
			delete e;
			return nullptr;
		}
		return e;
	}

	void ref_exec_destroy(void* h) { delete static_cast<RefExec*>(h); }

	int ref_exec_init(void* h)
	{
		RefExec& e = *static_cast<RefExec*>(h);
		try
		{
			sr::convert::to_helio(e.hd);
			auto& ip = e.interp;
			if (e.config.interp_planets)
			{
				ip = sr::interp::Interpolator(e.config, e.hd.planets, e.config.planet_history_file);
				while (ip.t1 <= e.t) ip.next(e.hd.planets);
				ip.cur_ts = 0;
				ip.n_ts = std::max<size_t>(1, static_cast<size_t>(std::round((ip.t1 - e.t) / e.config.dt)));
				ip.eff_dt = (ip.t1 - e.t) / static_cast<double>(ip.n_ts);
				ip.rel_t = e.t - ip.t0;
				ip.fill_one(e.hd.planets, ip.rel_t);
			}
			e.integ = sr::wh::WHIntegrator(e.hd.planets, e.hd.particles, e.config);
			// the reference uploads particle_a in its pre-partition order; the
			// fixtures start with no flagged particles, where both orders agree
			e.hd.particles.stable_partition_unflagged(0, e.hd.particles.n());
			size_t na = e.hd.particles.n_alive();
			e.hd.particles.stable_partition_alive(na, e.hd.particles.n() - na);
			e.dev_a = e.integ.particle_a;
			e.dev_n_alive = e.hd.particles.n_alive();
			e.swift = sr::swift::SwiftEncounterIntegrator(e.config, e.hd.particles.n());
			e.log << std::setprecision(17);   // as Executor::init sets encounter.out
			e.rb_r = e.hd.particles.r();
			e.rb_v = e.hd.particles.v();
			e.hd.planets_snapshot = e.hd.planets.base;
			update_planets(e);
		}
		catch (std::exception& ex)
		{
			e.err = ex.what();
			return -1;
		}
		return 0;
	}

	// One block of Executor::loop.
	int ref_exec_loop(void* h)
	{
		RefExec& e = *static_cast<RefExec*>(h);
		try
		{
			if (e.config.resolve_encounters)
			{
				loop_resolve(e);
				return 0;
			}
			auto& pa = e.hd.particles;
			size_t prev_alive = e.dev_n_alive;
			size_t presort = 0;
			if (e.dev_n_alive > 0)
			{
				for (size_t i = 0; i < e.dev_n_alive; i++)
				{
					uint32_t d = 0;
					sr::wh::MVSKernel::step_forward(pa.r()[i], pa.v()[i], pa.deathflags()[i], e.dev_a[i], d,
						e.dev_len, e.dev_npl, e.dev_h0_log.data(), e.dev_r_log.data(), e.dev_m.data(),
						e.dev_id.data(), e.dev_rh.data(), e.config.outer_radius, e.cur_dt, e.dev_m[0]);
					pa.deathtime_index()[i] = d;
				}
				if (!e.config.resolve_encounters)
				{
					for (size_t i = 0; i < e.dev_n_alive; i++)
					{
						uint16_t f = pa.deathflags()[i];
						if ((f & 0x01) == 0x01) f = static_cast<uint16_t>((f & 0xFF00) | 0x80);
						pa.deathflags()[i] = f;
					}
				}
				// stable partition of [0, n_alive) by flags == 0 (the device
				// partition is unstable; particles are compared by id)
				Vs idx(e.dev_n_alive);
				std::iota(idx.begin(), idx.end(), 0);
				auto mid = std::stable_partition(idx.begin(), idx.end(), [&](size_t k) { return pa.deathflags()[k] == 0; });
				presort = static_cast<size_t>(mid - idx.begin());
				pa.gather(idx, 0, e.dev_n_alive);
				gather(pa.deathtime_index(), idx, 0, e.dev_n_alive);
				gather(e.dev_a, idx, 0, e.dev_n_alive);
			}
			e.hd.planets_snapshot = e.hd.planets.base;
			e.t += e.cur_dt * static_cast<double>(e.cur_tbsize);
			update_planets(e);
			if (prev_alive > 0)
			{
				e.dev_n_alive = presort;
				pa.n_alive() = presort + pa.n_encounter();
				for (size_t i = e.dev_n_alive; i < prev_alive; i++)
				{
					pa.deathtime_map()[pa.id()[i]] = static_cast<float>(e.t);
					e.log << pa.id()[i] << ((pa.deathflags()[i] & 0x80) ? " death " : " encounter ") << e.t << "\n";
				}
			}
		}
		catch (std::exception& ex)
		{
			e.err = ex.what();
			return -1;
		}
		return 0;
	}

	void ref_exec_counts(void* h, size_t* n, size_t* n_alive, double* t, uint32_t* npl, uint32_t* log_len)
	{
		RefExec& e = *static_cast<RefExec*>(h);
		*n = e.hd.particles.n();
		*n_alive = e.dev_n_alive;
		*t = e.t;
		*npl = e.dev_npl;
		*log_len = e.dev_len;
	}

	const char* ref_exec_error(void* h) { return static_cast<RefExec*>(h)->err.c_str(); }

	// The SWIFT hand-offs made so far: count, then per call its arguments
	// (old-interval flag, t, rel_t, dt, prev/cur block lengths, first index,
	// particle count) and data (ids, state handed over, state and flags
	// end_integrate read back, all [n][3] / [n]).
	size_t ref_exec_swift_calls(void* h) { return static_cast<RefExec*>(h)->calls.size(); }

	void ref_exec_swift_call(void* h, size_t k, int* old, double* t3, size_t* sizes4)
	{
		const auto& c = static_cast<RefExec*>(h)->calls.at(k);
		*old = c.old;
		t3[0] = c.t; t3[1] = c.rel_t; t3[2] = c.dt;
		sizes4[0] = c.prev_len; sizes4[1] = c.cur_len; sizes4[2] = c.begin; sizes4[3] = c.n;
	}

	void ref_exec_swift_call_data(void* h, size_t k, uint32_t* ids, double* r_in, double* v_in, double* r_out,
		double* v_out, uint16_t* flags_out)
	{
		const auto& c = static_cast<RefExec*>(h)->calls.at(k);
		for (size_t i = 0; i < c.n; i++)
		{
			ids[i] = c.ids[i];
			flags_out[i] = c.flags_out[i];
			const f64_3* src[4] = { &c.r_in[i], &c.v_in[i], &c.r_out[i], &c.v_out[i] };
			double* dst[4] = { r_in, v_in, r_out, v_out };
			for (int q = 0; q < 4; q++)
			{
				dst[q][3 * i] = src[q]->x; dst[q][3 * i + 1] = src[q]->y; dst[q][3 * i + 2] = src[q]->z;
			}
		}
	}

	// stat.out as Executor::finish writes it (src/executor.cu:880-882)
	void ref_exec_write_stat(void* h, const char* path) { static_cast<RefExec*>(h)->swift.write_stat(path); }

	// counts in the reference's own terms: device n_alive, host n_alive
	// (alive + encounter), n_encounter
	void ref_exec_counts2(void* h, size_t* dev_alive, size_t* host_alive, size_t* n_encounter)
	{
		RefExec& e = *static_cast<RefExec*>(h);
		*dev_alive = e.dev_n_alive;
		*host_alive = e.hd.particles.n_alive();
		*n_encounter = e.hd.particles.n_encounter();
	}

	// encounter.out lines accumulated so far
	size_t ref_exec_encounter_log(void* h, char* buf, size_t cap)
	{
		std::string s = static_cast<RefExec*>(h)->log.str();
		if (buf && cap) { std::strncpy(buf, s.c_str(), cap - 1); buf[cap - 1] = 0; }
		return s.size();
	}

	void ref_exec_particles(void* h, double* r, double* v, double* a, uint32_t* id, uint16_t* flags, uint32_t* dti, double* deathtime)
	{
		RefExec& e = *static_cast<RefExec*>(h);
		auto& pa = e.hd.particles;
		for (size_t i = 0; i < pa.n(); i++)
		{
			r[3 * i] = pa.r()[i].x; r[3 * i + 1] = pa.r()[i].y; r[3 * i + 2] = pa.r()[i].z;
			v[3 * i] = pa.v()[i].x; v[3 * i + 1] = pa.v()[i].y; v[3 * i + 2] = pa.v()[i].z;
			f64_3 ai = i < e.dev_a.size() ? e.dev_a[i] : f64_3(0);
			a[3 * i] = ai.x; a[3 * i + 1] = ai.y; a[3 * i + 2] = ai.z;
			id[i] = pa.id()[i];
			flags[i] = pa.deathflags()[i];
			dti[i] = pa.deathtime_index()[i];
			auto it = pa.deathtime_map().find(pa.id()[i]);
			deathtime[i] = it == pa.deathtime_map().end() ? 0 : it->second;
		}
	}

	// The planet block the next ref_exec_loop call integrates with.
	void ref_exec_planet_block(void* h, double* r_log, double* h0_log, double* m, uint32_t* id, double* rh)
	{
		RefExec& e = *static_cast<RefExec*>(h);
		size_t nl = static_cast<size_t>(e.dev_len) * (e.dev_npl - 1);
		for (size_t i = 0; i < nl; i++)
		{
			r_log[3 * i] = e.dev_r_log[i].x; r_log[3 * i + 1] = e.dev_r_log[i].y; r_log[3 * i + 2] = e.dev_r_log[i].z;
		}
		for (size_t i = 0; i < e.dev_len; i++)
		{
			h0_log[3 * i] = e.dev_h0_log[i].x; h0_log[3 * i + 1] = e.dev_h0_log[i].y; h0_log[3 * i + 2] = e.dev_h0_log[i].z;
		}
		for (size_t i = 0; i < e.dev_npl; i++)
		{
			m[i] = e.dev_m[i];
			id[i] = e.dev_id[i];
			rh[i] = e.dev_rh[i];
		}
	}

	// Planet state at the end of the last completed block (the snapshot
	// the reference writes to dumps and tracks).
	void ref_exec_planets(void* h, size_t* n, double* m, double* r, double* v, uint32_t* id)
	{
		RefExec& e = *static_cast<RefExec*>(h);
		auto& p = e.hd.planets_snapshot;
		*n = p.n_alive;
		for (size_t i = 0; i < p.n_alive; i++)
		{
			m[i] = p.m[i];
			r[3 * i] = p.r[i].x; r[3 * i + 1] = p.r[i].y; r[3 * i + 2] = p.r[i].z;
			v[3 * i] = p.v[i].x; v[3 * i + 1] = p.v[i].y; v[3 * i + 2] = p.v[i].z;
			id[i] = p.id[i];
		}
	}

	// ---- format writers (golden files) ---------------------------------------

	// Writes the current state with save_data (binary or ASCII hybrid).
	int ref_exec_save_state(void* h, const char* path, int binary)
	{
		RefExec& e = *static_cast<RefExec*>(h);
		Configuration c = e.config;
		c.writesplit = false;
		c.writebinary = binary != 0;
		save_data(e.hd.planets_snapshot, e.hd.particles, c, path);
		return 0;
	}

	int ref_exec_write_track(void* h, const char* path, int append, int bary)
	{
		RefExec& e = *static_cast<RefExec*>(h);
		std::ofstream out(path, append ? (std::ios_base::binary | std::ios_base::app) : std::ios_base::binary);
		HostParticleSnapshot snap = e.hd.particles.base;
		snap.sort_by_id(0, snap.n_alive);
		save_binary_track(out, e.hd.planets_snapshot, snap, e.t, true, bary != 0);
		return 0;
	}

	int ref_exec_write_plhist(void* h, const char* path, int begin)
	{
		RefExec& e = *static_cast<RefExec*>(h);
		std::ofstream out(path, begin ? std::ios_base::binary : (std::ios_base::binary | std::ios_base::app));
		if (begin) begin_swift_plhist(out, e.hd.planets_snapshot);
		save_swift_plhist(out, e.hd.planets_snapshot, e.t);
		return 0;
	}

	int ref_write_config(const char* config_text, const char* path)
	{
		Configuration c;
		std::istringstream in(config_text);
		try { read_configuration(in, &c); } catch (std::exception&) { return -1; }
		std::ofstream out(path);
		write_configuration(out, c);
		return 0;
	}

	// Returns 0 if the text parses and validates, else -1 with the message.
	int ref_check_config(const char* config_text, char* msg, size_t cap)
	{
		Configuration c;
		std::istringstream in(config_text);
		try { read_configuration(in, &c); }
		catch (std::exception& ex)
		{
			if (msg && cap) { std::strncpy(msg, ex.what(), cap - 1); msg[cap - 1] = 0; }
			return -1;
		}
		return 0;
	}
}
