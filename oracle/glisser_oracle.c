/*
 * glisser oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference (skkestrel/glisser) algorithms on the
 * massless-particle Wisdom-Holman / MVS time-block path.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, as the
 * checker or as the timed CPU baseline; the product never links or calls it.
 *
 * Parity is pinned: tests/golden/ holds vectors produced by the unmodified
 * reference sources (built by oracle/build_ref.sh, driven by
 * tests/golden/make_golden.py), and tests/test_oracle_pin.py checks this file
 * against them.  Compile with -ffp-contract=off so that the arithmetic is the
 * same on x86-64 and aarch64 hosts.
 *
 * Each function names the reference file:line it follows.  The floating-point
 * expressions keep the reference's evaluation order on purpose: the oracle is
 * meant to reproduce the reference's numbers, not to improve them.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846

typedef struct { double x, y, z; } v3;

static inline v3 mk(double x, double y, double z) { v3 r = { x, y, z }; return r; }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 scl(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 dvs(v3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline double lensq(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline v3 ld(const double* p, size_t i) { return mk(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
static inline void st(double* p, size_t i, v3 a) { p[3 * i] = a.x; p[3 * i + 1] = a.y; p[3 * i + 2] = a.z; }

/* number of whole orbits removed from a drift: the reference writes
 * (int)(dt*n/M_2PI) with M_2PI expanding to `M_PI * 2` unparenthesised
 * (src/types.h:8, src/wh.cu:91), which evaluates as (dt*n/M_PI)*2. */
static inline double orbits_removed(double dtn) { return (ORC_PI * 2) * (int) (dtn / ORC_PI * 2); }

/* ------------------------------------------------------------------------ */
/* Reference GPU particle kernel: MVSKernel (src/wh.cu:43-177)              */
/* ------------------------------------------------------------------------ */

/* src/wh.cu:43-72 -- five fixed Newton iterations; the flag word is
 * overwritten with the non-convergence bit (quirk: clobbers 0x08). */
static void mvs_kepeq(double dM, double ecosEo, double esinEo, double* dE, double* sindE, double* cosdE, uint16_t* flags)
{
	double f, fp, delta = 0;
	*sindE = sin(*dE);
	*cosdE = cos(*dE);
	for (int i = 0; i < 5; i++)
	{
		f = *dE - ecosEo * (*sindE) + esinEo * (1. - *cosdE) - dM;
		fp = 1. - ecosEo * (*cosdE) + esinEo * (*sindE);
		delta = -f / fp;
		*dE += delta;
		*sindE = sin(*dE);
		*cosdE = cos(*dE);
	}
	*flags = (uint16_t) ((fabs(delta) > 1e-14) << 2);
}

/* src/wh.cu:75-110 -- elliptic heliocentric drift through f and g. */
static void mvs_drift(v3* r, v3* v, uint16_t* flags, double dt, double mu)
{
	double dist = sqrt(lensq(*r));
	double vdotr = v->x * r->x + v->y * r->y + v->z * r->z;
	double energy = lensq(*v) * 0.5 - mu / dist;
	*flags = (uint16_t) ((energy >= 0) << 3);
	double a = -0.5 * mu / energy;
	double n_ = sqrt(mu / (a * a * a));
	double ecosEo = 1.0 - dist / a;
	double esinEo = vdotr / (n_ * a * a);
	double dM = dt * n_ - orbits_removed(dt * n_);
	double _dt = dM / n_;
	double dE = dM - esinEo + esinEo * cos(dM) + ecosEo * sin(dM);
	double sindE, cosdE;
	mvs_kepeq(dM, ecosEo, esinEo, &dE, &sindE, &cosdE, flags);
	double fp = 1.0 - ecosEo * cosdE + esinEo * sindE;
	double f = 1.0 + a * (cosdE - 1.0) / dist;
	double g = _dt + (sindE - dE) / n_;
	double fdot = -n_ * sindE * a / (dist * fp);
	double gdot = 1.0 + (cosdE - 1.0) / fp;
	v3 r0 = *r;
	*r = add(scl(r0, f), scl(*v, g));
	*v = add(scl(r0, fdot), scl(*v, gdot));
}

/* The particle drift used by orc_block: 0 = reference MVS elliptic drift
 * (src/wh.cu:75-110), 1 = universal-variable drift through the reference's
 * kepu (src/wh.cpp:836-852, kepu at :399-420). */
static void uv_drift(v3* r, v3* v, uint16_t* flags, double dt, double mu);

/* src/wh.cu:113-177 -- one time block for one particle.  planet_n counts
 * the Sun; r_log is [tbsize][planet_n-1][3]. */
static void block_one(int drift_kind, v3* r, v3* v, uint16_t* flags, v3* a, uint32_t* deathtime_index,
	uint32_t tbsize, uint32_t planet_n, const double* h0_log, const double* r_log,
	const double* m, const uint32_t* pl_id, const double* rh, double outer_radius, double dt, double mu)
{
	*deathtime_index = 0;
	for (uint32_t step = 0; step < tbsize; step++)
	{
		if (*flags != 0) continue;
		*v = add(*v, scl(*a, dt / 2));
		if (drift_kind == 0) mvs_drift(r, v, flags, dt, mu);
		else uv_drift(r, v, flags, dt, mu);
		*a = ld(h0_log, step);
		for (uint32_t i = 1; i < planet_n; i++)
		{
			v3 dr = sub(*r, ld(r_log, (size_t) step * (planet_n - 1) + i - 1));
			double rad = lensq(dr);
			if (rad < rh[i] * rh[i] && *flags == 0)
				*flags = (uint16_t) ((pl_id[i] << 8) | 0x0001);
			double inv3 = 1. / (rad * sqrt(rad));
			double fac = m[i] * inv3;
			*a = sub(*a, scl(dr, fac));
		}
		double rad = lensq(*r);
		if (rad < rh[0] * rh[0]) *flags = 0x0001;
		if (rad > outer_radius * outer_radius) *flags = 0x0002;
		*v = add(*v, scl(*a, dt / 2));
		*deathtime_index = step + 1;
	}
}

/* Vectors are [n][3]. */
void orc_block(int drift_kind, size_t n, double* r, double* v, double* a, uint16_t* flags, uint32_t* dti,
	uint32_t tbsize, uint32_t planet_n, const double* h0_log, const double* r_log,
	const double* m, const uint32_t* pl_id, const double* rh, double outer_r, double dt, double mu)
{
	for (size_t i = 0; i < n; i++)
	{
		v3 ri = ld(r, i), vi = ld(v, i), ai = ld(a, i);
		block_one(drift_kind, &ri, &vi, &flags[i], &ai, &dti[i], tbsize, planet_n, h0_log, r_log, m, pl_id, rh, outer_r, dt, mu);
		st(r, i, ri);
		st(v, i, vi);
		st(a, i, ai);
	}
}

/* ------------------------------------------------------------------------ */
/* Universal-variable Kepler solver: src/wh.cpp:131-420 (SWIFT drift_kepu*) */
/* ------------------------------------------------------------------------ */

#define DANBYB 1e-13

/* src/wh.cpp:131-173 */
static int kepu_p3solve(double dt, double r0, double mu, double alpha, double u, double* s)
{
	double denom = (mu - alpha * r0) / 6.;
	double a2 = 0.5 * u / denom;
	double a1 = r0 / denom;
	double a0 = -dt / denom;
	double q = (a1 - a2 * a2 / 3.) / 3.;
	double r = (a1 * a2 - 3. * a0) / 6. - (a2 * a2 * a2) / 27.;
	double sq2 = q * q * q + r * r;
	if (sq2 >= 0)
	{
		double sq = sqrt(sq2), p1, p2;
		if (r + sq <= 0) p1 = -pow(-r - sq, 1. / 3.);
		else p1 = pow(r + sq, 1. / 3.);
		if (r - sq <= 0) p2 = -pow(-r + sq, 1. / 3.);
		else p2 = pow(r - sq, 1. / 3.);
		*s = p1 + p2 - a2 / 3.;
		return 0;
	}
	*s = 0;
	return 1;
}

/* src/wh.cpp:188-220 */
void orc_kepu_guess(double dt, double r0, double mu, double alpha, double u, double* s)
{
	if (alpha > 0)
	{
		if (dt / r0 <= 0.4)
		{
			*s = dt / r0 - (dt * dt * u) / (2. * r0 * r0 * r0);
		}
		else
		{
			double a = mu / alpha;
			double en = sqrt(mu / (a * a * a));
			double ec = 1.0 - r0 / a;
			double es = u / (en * a * a);
			double e = sqrt(ec * ec + es * es);
			double y = en * dt - es;
			double sy = sin(y), cy = cos(y);
			double sigma = es * cy + ec * sy > 0 ? 1 : -1;
			double x = y + sigma * .85 * e;
			*s = x / sqrt(alpha);
		}
	}
	else
	{
		if (kepu_p3solve(dt, r0, mu, alpha, u, s)) *s = dt / r0;
	}
}

/* src/wh.cpp:230-257 (Danby p.172 eq. 6.9.15) */
static void kepu_stumpff(double x, double* c0, double* c1, double* c2, double* c3)
{
	uint32_t n = 0;
	double xm = 0.1;
	while (fabs(x) >= xm)
	{
		n++;
		x /= 4.;
	}
	*c2 = (1. - x * (1. - x * (1. - x * (1. - x * (1. - x * (1. - x / 182.) / 132.) / 90.) / 56.) / 30.) / 12.) / 2.;
	*c3 = (1. - x * (1. - x * (1. - x * (1. - x * (1. - x * (1. - x / 210.) / 156.) / 110.) / 72.) / 42.) / 20.) / 6.;
	*c1 = 1. - x * *c3;
	*c0 = 1. - x * *c2;
	for (uint32_t i = 0; i < n; i++)
	{
		*c3 = (*c2 + *c0 * *c3) / 4.;
		*c2 = *c1 * *c1 / 2.;
		*c1 = *c0 * *c1;
		*c0 = 2. * *c0 * *c0 - 1.;
		x *= 4;
	}
}

/* Checker option, off by default (then the reference's arithmetic): on
 * acceptance, evaluate the G-functions at the s that the accepting pass
 * corrected to, not at the s whose residual passed, so that each drift is
 * converged to O(DANBYB^2) instead of carrying up to DANBYB of dt.  For
 * comparisons on workloads with few steps per orbit, where the reference's
 * per-drift residual accumulates above the parity tolerance. */
static int g_kepu_converged = 0;
void orc_set_kepu_converged(int on) { g_kepu_converged = on; }

static void kepu_at(double s, double mu, double alpha, double r0, double u, double* fp, double* c1, double* c2,
	double* c3)
{
	double c0;
	kepu_stumpff(s * s * alpha, &c0, c1, c2, c3);
	*c1 = *c1 * s;
	*c2 = *c2 * s * s;
	*c3 = *c3 * s * s * s;
	*fp = r0 * c0 + u * *c1 + mu * *c2;
}

/* src/wh.cpp:260-290; *iters receives the number of passes */
static int kepu_new(double s, double dt, double r0, double mu, double alpha, double u,
	double* fp, double* c1, double* c2, double* c3, int* iters)
{
	for (int nc = 0; nc < 7; nc++)
	{
		double x = s * s * alpha;
		double c0;
		kepu_stumpff(x, &c0, c1, c2, c3);
		*c1 = *c1 * s;
		*c2 = *c2 * s * s;
		*c3 = *c3 * s * s * s;
		double f = r0 * *c1 + u * *c2 + mu * *c3 - dt;
		*fp = r0 * c0 + u * *c1 + mu * *c2;
		double fpp = (-r0 * alpha + mu) * *c1 + u * c0;
		double fppp = (-r0 * alpha + mu) * c0 - u * alpha * *c1;
		double ds = -f / *fp;
		ds = -f / (*fp + ds * fpp / 2.);
		ds = -f / (*fp + ds * fpp / 2. + ds * ds * fppp / 6.);
		s = s + ds;
		double fdt = f / dt;
		if (iters) *iters = nc + 1;
		if (fdt * fdt < DANBYB * DANBYB)
		{
			if (g_kepu_converged) kepu_at(s, mu, alpha, r0, u, fp, c1, c2, c3);
			return 0;
		}
	}
	return 1;
}

/* src/wh.cpp:306-316 */
static double kepu_fchk(double dt, double r0, double mu, double alpha, double u, double s)
{
	double c0, c1, c2, c3;
	double x = s * s * alpha;
	kepu_stumpff(x, &c0, &c1, &c2, &c3);
	c1 = c1 * s;
	c2 = c2 * s * s;
	c3 = c3 * s * s * s;
	return r0 * c1 + u * c2 + mu * c3 - dt;
}

/* src/wh.cpp:340-382 (keeps SWIFT's `-40.*alpha` in f'') */
static int kepu_lag(double s, double dt, double r0, double mu, double alpha, double u,
	double* fp, double* c1, double* c2, double* c3)
{
	uint32_t ncmax = 400;
	double ln = 5.0;
	for (uint32_t nc = 0; nc <= ncmax; nc++)
	{
		double c0;
		double x = s * s * alpha;
		kepu_stumpff(x, &c0, c1, c2, c3);
		*c1 = *c1 * s;
		*c2 = *c2 * s * s;
		*c3 = *c3 * s * s * s;
		double f = r0 * *c1 + u * *c2 + mu * *c3 - dt;
		*fp = r0 * c0 + u * *c1 + mu * *c2;
		double fpp = (-40. * alpha + mu) * *c1 + u * c0;
		double ds = -ln * f / (*fp + (*fp > 0 ? 1 : -1) * sqrt(fabs((ln - 1.) * (ln - 1.) * *fp * *fp - (ln - 1.) * ln * f * fpp)));
		s = s + ds;
		double fdt = f / dt;
		if (fdt * fdt < DANBYB * DANBYB)
		{
			if (g_kepu_converged) kepu_at(s, mu, alpha, r0, u, fp, c1, c2, c3);
			return 0;
		}
	}
	return 1;
}

/* src/wh.cpp:399-420.  Returns nonzero on failure.  *iters (optional)
 * receives the Newton passes, or 100 when Laguerre's method was needed. */
int orc_kepu(double dt, double r0, double mu, double alpha, double u,
	double* fp, double* c1, double* c2, double* c3, int* iters)
{
	double s;
	orc_kepu_guess(dt, r0, mu, alpha, u, &s);
	double st = s;
	if (kepu_new(s, dt, r0, mu, alpha, u, fp, c1, c2, c3, iters))
	{
		double fo = kepu_fchk(dt, r0, mu, alpha, u, st);
		double fn = kepu_fchk(dt, r0, mu, alpha, u, s);
		if (fabs(fo) < fabs(fn)) s = st;
		if (iters) *iters = 100;
		return kepu_lag(s, dt, r0, mu, alpha, u, fp, c1, c2, c3);
	}
	return 0;
}

/* src/wh.cpp:836-852 applied to every orbit (the hyperbolic branch of
 * drift_single), with the GPU kernel's flag convention: 0x08 when the orbit
 * is unbound, 0x04 when kepu fails. */
static void uv_drift(v3* r, v3* v, uint16_t* flags, double dt, double mu)
{
	double dist = sqrt(lensq(*r));
	double vsq = lensq(*v);
	double vdotr = v->x * r->x + v->y * r->y + v->z * r->z;
	double energy = vsq;
	energy *= 0.5;
	energy -= mu / dist;
	double fp, c1, c2, c3;
	int fail = orc_kepu(dt, dist, mu, -2 * energy, vdotr, &fp, &c1, &c2, &c3, NULL);
	*flags = (uint16_t) (((energy >= 0) << 3) | (fail << 2));
	double f = 1.0 - (mu / dist) * c2;
	double g = dt - mu * c3;
	double fdot = -(mu / (fp * dist)) * c1;
	double gdot = 1. - (mu / fp) * c2;
	v3 r0 = *r, v0 = *v;
	*r = add(scl(r0, f), scl(v0, g));
	*v = add(scl(r0, fdot), scl(v0, gdot));
}

/* Full universal-variable drift of [n][3] states (used to check the device
 * drift per solve).  iters receives kepu's pass count per particle. */
void orc_uv_drift(size_t n, double* r, double* v, uint16_t* flags, double dt, double mu, int* iters)
{
	for (size_t i = 0; i < n; i++)
	{
		v3 ri = ld(r, i), vi = ld(v, i);
		double dist = sqrt(lensq(ri));
		double vsq = lensq(vi);
		double vdotr = vi.x * ri.x + vi.y * ri.y + vi.z * ri.z;
		double energy = vsq;
		energy *= 0.5;
		energy -= mu / dist;
		double fp, c1, c2, c3;
		int it = 0;
		int fail = orc_kepu(dt, dist, mu, -2 * energy, vdotr, &fp, &c1, &c2, &c3, &it);
		if (iters) iters[i] = it;
		flags[i] = (uint16_t) (((energy >= 0) << 3) | (fail << 2));
		double f = 1.0 - (mu / dist) * c2;
		double g = dt - mu * c3;
		double fdot = -(mu / (fp * dist)) * c1;
		double gdot = 1. - (mu / fp) * c2;
		st(r, i, add(scl(ri, f), scl(vi, g)));
		st(v, i, add(scl(ri, fdot), scl(vi, gdot)));
	}
}

/* ------------------------------------------------------------------------ */
/* Orbital elements: src/convert.cpp:182-497 (SWIFT orbel_*)                */
/* ------------------------------------------------------------------------ */

/* src/convert.cpp:183-222 */
static double ehie(double e, double m)
{
	int iflag = 0;
	int nper = (int) (m / (2 * ORC_PI));
	m = m - nper * 2 * ORC_PI;
	if (m < 0) m += 2 * ORC_PI;
	if (m > ORC_PI)
	{
		m = 2 * ORC_PI - m;
		iflag = 1;
	}
	double x = pow(6 * m, 1. / 3) - m;
	for (int i = 0; i < 3; i++)
	{
		double sa = sin(x + m);
		double ca = cos(x + m);
		double esa = e * sa;
		double eca = e * ca;
		double f = x - esa;
		double fp = 1 - eca;
		double dx = -f / fp;
		dx = -f / (fp + dx * esa / 2);
		dx = -f / (fp + dx * (esa + eca * dx / 3) / 2);
		x = x + dx;
	}
	if (iflag) return 2 * ORC_PI - m - x;
	return m + x;
}

/* src/convert.cpp:224-248 */
static double eget(double e, double m, int n)
{
	double sm = sin(m);
	double cm = cos(m);
	double x = m + e * sm * (1 + e * (cm + e * (1 - 1.5 * sm * sm)));
	for (int i = 0; i < n; i++)
	{
		double sx = sin(x);
		double cx = cos(x);
		double es = e * sx;
		double ec = e * cx;
		double f = x - es - m;
		double fp = 1 - ec;
		double fpp = es;
		double fppp = ec;
		double dx = -f / fp;
		dx = -f / (fp + dx * fpp / 2);
		dx = -f / (fp + dx * fpp / 2 + dx * dx * fppp / 6);
		x = x + dx;
	}
	return x;
}

/* src/convert.cpp:250-255 */
static double ehybrid(double e, double m)
{
	if (e < 0.18) return eget(e, m, 1);
	else if (e < 0.8) return eget(e, m, 2);
	return ehie(e, m);
}

/* src/convert.cpp:277-335 */
void orc_from_elements(double mu, double a, double e, double i, double capom, double om, double f, double* rout, double* vout)
{
	double prec = 1.0e-13;
	double u = om + f;
	double xhat = cos(u) * cos(capom) - cos(i) * sin(capom) * sin(u);
	double yhat = cos(u) * sin(capom) + cos(i) * cos(capom) * sin(u);
	double zhat = sin(i) * sin(u);
	double hx = sin(capom) * sin(i);
	double hy = -cos(capom) * sin(i);
	double hz = cos(i);
	double r, h;
	if (fabs(e - 1.0) > prec)
	{
		r = a * (1.0 - e * e) / (1.0 + e * cos(f));
		h = sqrt(mu * a * (1.0 - e * e));
	}
	else
	{
		h = sqrt(2.0 * mu * a);
		r = a / (cos(f / 2.0) * cos(f / 2.0));
	}
	rout[0] = r * xhat;
	rout[1] = r * yhat;
	rout[2] = r * zhat;
	double thx = hy * zhat - hz * yhat;
	double thy = hz * xhat - hx * zhat;
	double thz = hx * yhat - hy * xhat;
	double thdot = h / (r * r);
	double rdot = e * mu * sin(f) / h;
	vout[0] = r * thdot * thx + rdot * xhat;
	vout[1] = r * thdot * thy + rdot * yhat;
	vout[2] = r * thdot * thz + rdot * zhat;
}

/* src/convert.cpp:257-275 */
void orc_from_elements_M(double mu, double a, double e, double i, double capom, double om, double M, double* r, double* v)
{
	double E = ehybrid(e, M);
	double f = acos((cos(E) - e) / (1 - e * cos(E)));
	E = E - (int) (E / 2 / ORC_PI) * 2 * ORC_PI;
	if (E > ORC_PI) E -= 2 * ORC_PI;
	else if (E < -ORC_PI) E += 2 * ORC_PI;
	if (E < 0) f = -f;
	orc_from_elements(mu, a, e, i, capom, om, f, r, v);
}

/* orc_from_elements_M over n element rows (a, e, i, capom, om, M) into [n][3]
 * r and v: the particle generator of targets/make_state.cpp:126-165 without its
 * RNG, for callers that must not load the product library. */
void orc_elements_to_cartesian(size_t n, double mu, const double* el, double* r, double* v)
{
	for (size_t k = 0; k < n; k++)
	{
		const double* e = el + 6 * k;
		orc_from_elements_M(mu, e[0], e[1], e[2], e[3], e[4], e[5], r + 3 * k, v + 3 * k);
	}
}

/* src/convert.cpp:337-490; out6 = a, e, i, capom, om, f */
void orc_to_elements(double mu, const double* rr_, const double* vv_, int* esignout, double* out6)
{
	double a = 0, e = 0, i = 0, capom = 0, om = 0, f = 0;
	int esign;
	double x = rr_[0], y = rr_[1], z = rr_[2];
	double vx = vv_[0], vy = vv_[1], vz = vv_[2];
	double pi = 2.0 * asin(1.0);
	double prec = 1.0e-13;
	double hx = y * vz - z * vy;
	double hy = z * vx - x * vz;
	double hz = x * vy - y * vx;
	double hsq = hx * hx + hy * hy + hz * hz;
	if (hsq > prec)
	{
		i = acos(hz / sqrt(hsq));
		if (fabs(i) < prec) capom = 0.0;
		else if (fabs(pi - fabs(i)) < prec) capom = 0.0;
		else capom = atan2(hx, -hy);
		double vsq = vx * vx + vy * vy + vz * vz;
		double vdotr = x * vx + y * vy + z * vz;
		double rr = sqrt(x * x + y * y + z * z);
		double xhat = x / rr, yhat = y / rr, zhat = z / rr;
		double nx = cos(capom), ny = sin(capom);
		double fac = vsq * rr - mu;
		double Px = fac * xhat - vdotr * vx;
		double Py = fac * yhat - vdotr * vy;
		double Pz = fac * zhat - vdotr * vz;
		double modP = sqrt(Px * Px + Py * Py + Pz * Pz);
		e = modP / mu;
		if (fabs(e) < prec) om = 0.0;
		else
		{
			if ((i < prec) || (pi - i < prec)) om = atan2(Py, Px);
			else
			{
				double ecosw = (nx * Px + ny * Py) / mu;
				om = acos(ecosw / e);
				if (fabs(Pz) > prec) om *= fabs(Pz) / Pz;
			}
		}
		double energy = vsq / 2.0 - mu / rr;
		if (fabs(energy) < prec)
		{
			esign = 0;
			a = 0.5 * hsq / mu;
			if (fabs(vdotr) < prec) f = 0.0;
			else f = 2.0 * acos(sqrt(a / rr)) * vdotr / fabs(vdotr);
		}
		else if (energy > 0.0)
		{
			esign = 1;
			a = -0.5 * mu / energy;
			if (fabs(vdotr) < prec) f = 0.0;
			else
			{
				fac = a * (1.0 - e * e) / rr - 1.0;
				f = acos(fac / e) * vdotr / fabs(vdotr);
			}
		}
		else
		{
			esign = -1;
			a = -0.5 * mu / energy;
			if (fabs(e) > prec)
			{
				if (fabs(vdotr) < prec)
				{
					f = rr < a ? 0.0 : pi;
				}
				else
				{
					fac = a * (1.0 - e * e) / rr - 1.0;
					f = acos(fac / e) * vdotr / fabs(vdotr);
					if (isnan(f)) f = rr < a ? 0.0 : pi;
				}
			}
			else
			{
				fac = (x * nx + y * ny) / rr;
				f = acos(fac);
				if (fabs(z) > prec) f *= fabs(z) / z;
				else if ((i < prec) || (pi - i < prec)) f = atan2(y, x) * cos(i);
			}
		}
	}
	else
	{
		esign = 1;
		a = sqrt(x * x + y * y + z * z);
		e = HUGE_VAL;
		i = asin(z / sqrt(x * x + y * y + z * z));
		capom = atan2(y, x);
		om = HUGE_VAL;
		f = HUGE_VAL;
	}
	if (esignout) *esignout = esign;
	out6[0] = a; out6[1] = e; out6[2] = i; out6[3] = capom; out6[4] = om; out6[5] = f;
}

/* src/convert.cpp:492-497 */
double orc_mean_anomaly(double e, double f)
{
	double E = acos((e + cos(f)) / (1 + e * cos(f)));
	if (f < 0) E = -E;
	return E - e * sin(E);
}

/* ------------------------------------------------------------------------ */
/* Planet Wisdom-Holman integrator: src/wh.cpp:19-43, 472-1067,             */
/* src/convert.cpp:9-122                                                    */
/* ------------------------------------------------------------------------ */

typedef struct
{
	size_t n;          /* planets including the Sun */
	double* m;
	v3* r;             /* heliocentric */
	v3* v;
	uint32_t* id;
	double* eta;
	v3 *rj, *vj, *acc;
	double *ihc, *ijc, *pmu;
	double* rh;
	double cull_radius, esf;
} orc_planets;

/* src/wh.cpp:19-43 (adaptive, MAXKEP=10); returns 1 when unconverged */
static int kepeq_adaptive(double dM, double esinEo, double ecosEo, double* dE, double* sindE, double* cosdE)
{
	double f, fp, delta;
	*sindE = sin(*dE);
	*cosdE = cos(*dE);
	for (int i = 0; i < 10; i++)
	{
		f = *dE - ecosEo * (*sindE) + esinEo * (1. - *cosdE) - dM;
		fp = 1. - ecosEo * (*cosdE) + esinEo * (*sindE);
		delta = -f / fp;
		if (fabs(delta) < 1e-14) return 0;
		*dE += delta;
		*sindE = sin(*dE);
		*cosdE = cos(*dE);
	}
	return 1;
}

/* src/convert.cpp:101-122 */
static void helio_to_jacobi_r(orc_planets* p)
{
	p->rj[0] = mk(0, 0, 0);
	p->rj[1] = p->r[1];
	v3 sum = mk(0, 0, 0);
	for (size_t i = 2; i < p->n; i++)
	{
		sum = add(sum, scl(p->r[i - 1], p->m[i - 1]));
		v3 bary = dvs(sum, p->eta[i - 1]);
		p->rj[i] = sub(p->r[i], bary);
	}
}

/* src/convert.cpp:75-99 */
static void helio_to_jacobi_v(orc_planets* p)
{
	p->vj[0] = mk(0, 0, 0);
	p->vj[1] = p->v[1];
	v3 psum = mk(0, 0, 0);
	for (size_t i = 2; i < p->n; i++)
	{
		psum = add(psum, scl(p->v[i - 1], p->m[i - 1]));
		v3 vsum = dvs(psum, p->eta[i - 1]);
		p->vj[i] = sub(p->v[i], vsum);
	}
}

/* src/convert.cpp:9-28 */
static void jacobi_to_helio(orc_planets* p)
{
	p->r[0] = mk(0, 0, 0);
	p->v[0] = mk(0, 0, 0);
	p->r[1] = p->rj[1];
	p->v[1] = p->vj[1];
	v3 rsum = mk(0, 0, 0), vsum = mk(0, 0, 0);
	for (size_t i = 2; i < p->n; i++)
	{
		rsum = add(rsum, scl(p->rj[i - 1], p->m[i - 1] / p->eta[i - 1]));
		vsum = add(vsum, scl(p->vj[i - 1], p->m[i - 1] / p->eta[i - 1]));
		p->r[i] = add(p->rj[i], rsum);
		p->v[i] = add(p->vj[i], vsum);
	}
}

/* src/wh.cpp:696-756; writes h0 for this step into *h0 */
static void helio_acc_planets(orc_planets* p, v3* h0)
{
	size_t n = p->n;
	for (size_t i = 1; i < n; i++)
	{
		double r2 = lensq(p->r[i]);
		p->ihc[i] = 1. / (sqrt(r2) * r2);
		r2 = lensq(p->rj[i]);
		p->ijc[i] = 1. / (sqrt(r2) * r2);
	}
	v3 a_common = mk(0, 0, 0);
	for (size_t i = 2; i < n; i++)
	{
		double mfac = p->m[i] * p->ihc[i];
		a_common = sub(a_common, scl(p->r[i], mfac));
	}
	for (size_t i = 1; i < n; i++) p->acc[i] = a_common;
	*h0 = sub(a_common, scl(scl(p->r[1], p->m[1]), p->ihc[1]));
	for (size_t i = 2; i < n; i++)
		p->acc[i] = add(p->acc[i], scl(sub(scl(p->rj[i], p->ijc[i]), scl(p->r[i], p->ihc[i])), p->m[0]));
	v3 a_accum = mk(0, 0, 0);
	for (size_t i = 2; i < n; i++)
	{
		double mfac = p->m[i] * p->m[0] * p->ijc[i] / p->eta[i - 1];
		a_accum = add(a_accum, scl(p->rj[i], mfac));
		p->acc[i] = add(p->acc[i], a_accum);
	}
	for (size_t i = 1; i + 1 < n; i++)
	{
		for (size_t j = i + 1; j < n; j++)
		{
			v3 dr = sub(p->r[j], p->r[i]);
			double r2 = lensq(dr);
			double irij3 = 1. / (r2 * sqrt(r2));
			double mfac = p->m[i] * irij3;
			p->acc[j] = sub(p->acc[j], scl(dr, mfac));
			mfac = p->m[j] * irij3;
			p->acc[i] = add(p->acc[i], scl(dr, mfac));
		}
	}
}

/* src/wh.cpp:472-495 */
static void recalculate_rh(orc_planets* p)
{
	if (fabs(p->esf) > 1e-6)
	{
		p->rh[0] = p->cull_radius;
		for (size_t i = 1; i < p->n; i++)
		{
			double el[6];
			double rr[3] = { p->r[i].x, p->r[i].y, p->r[i].z };
			double vv[3] = { p->v[i].x, p->v[i].y, p->v[i].z };
			orc_to_elements(p->m[0] + p->m[i], rr, vv, NULL, el);
			p->rh[i] = p->esf * el[0] * (1 - el[1]) * pow(p->m[i] / (3 * p->m[0]), 1. / 3);
		}
	}
	else
	{
		for (size_t i = 0; i < p->n; i++) p->rh[i] = p->cull_radius;
	}
}

/* src/wh.cpp:875-957 with fixediterations = false; returns nonzero on an
 * unbound or unconverged Jacobi orbit (the reference throws). */
static int drift_planets(orc_planets* p, double t)
{
	for (size_t i = 1; i < p->n; i++)
	{
		v3 r0 = p->rj[i], v0 = p->vj[i];
		double dist = sqrt(lensq(r0));
		double energy = lensq(v0);
		double vdotr = v0.x * r0.x + v0.y * r0.y + v0.z * r0.z;
		energy *= 0.5;
		energy -= p->pmu[i] / dist;
		if (energy >= 0) return 1;
		double a = -0.5 * p->pmu[i] / energy;
		double n_ = sqrt(p->pmu[i] / (a * a * a));
		double ecosEo = 1.0 - dist / a;
		double esinEo = vdotr / (n_ * a * a);
		double dM = t * n_ - orbits_removed(t * n_);
		double adv_dt = dM / n_;
		double dE = dM - esinEo + esinEo * cos(dM) + ecosEo * sin(dM);
		double sindE, cosdE;
		if (kepeq_adaptive(dM, esinEo, ecosEo, &dE, &sindE, &cosdE)) return 2;
		double fp = 1.0 - ecosEo * cosdE + esinEo * sindE;
		double f = 1.0 + a * (cosdE - 1.0) / dist;
		double g = adv_dt + (sindE - dE) / n_;
		double fdot = -n_ * sindE * a / (dist * fp);
		double gdot = 1.0 + (cosdE - 1.0) / fp;
		p->rj[i] = add(scl(r0, f), scl(v0, g));
		p->vj[i] = add(scl(r0, fdot), scl(v0, gdot));
	}
	return 0;
}

/* src/wh.cpp:1027-1067; appends r[1..n) to r_log and h0 to *h0 */
static int step_planets(orc_planets* p, double dt, double* r_log_step, v3* h0)
{
	for (size_t i = 1; i < p->n; i++) p->v[i] = add(p->v[i], scl(p->acc[i], dt / 2));
	helio_to_jacobi_v(p);
	for (size_t i = 1; i < p->n; i++) p->pmu[i] = p->m[0] * p->eta[i] / p->eta[i - 1];
	int err = drift_planets(p, dt);
	if (err) return err;
	jacobi_to_helio(p);
	helio_acc_planets(p, h0);
	for (size_t i = 1; i < p->n; i++) st(r_log_step, i - 1, p->r[i]);
	for (size_t i = 1; i < p->n; i++) p->v[i] = add(p->v[i], scl(p->acc[i], dt / 2));
	return 0;
}

static orc_planets* planets_new(size_t n)
{
	orc_planets* p = (orc_planets*) calloc(1, sizeof(orc_planets));
	p->n = n;
	p->m = (double*) calloc(n, sizeof(double));
	p->r = (v3*) calloc(n, sizeof(v3));
	p->v = (v3*) calloc(n, sizeof(v3));
	p->id = (uint32_t*) calloc(n, sizeof(uint32_t));
	p->eta = (double*) calloc(n, sizeof(double));
	p->rj = (v3*) calloc(n, sizeof(v3));
	p->vj = (v3*) calloc(n, sizeof(v3));
	p->acc = (v3*) calloc(n, sizeof(v3));
	p->ihc = (double*) calloc(n, sizeof(double));
	p->ijc = (double*) calloc(n, sizeof(double));
	p->pmu = (double*) calloc(n, sizeof(double));
	p->rh = (double*) calloc(n, sizeof(double));
	return p;
}

static void planets_free(orc_planets* p)
{
	if (!p) return;
	free(p->m); free(p->r); free(p->v); free(p->id); free(p->eta); free(p->rj); free(p->vj);
	free(p->acc); free(p->ihc); free(p->ijc); free(p->pmu); free(p->rh); free(p);
}

/* ------------------------------------------------------------------------ */
/* Planetary-history interpolation: src/interp.cpp:13-293                   */
/* ------------------------------------------------------------------------ */

typedef struct
{
	FILE* in;
	size_t cap;               /* Planet-History-Max-Planet-Count */
	double user_dt;
	double sun_m;
	double t0, t1, t_m1, eff_dt, rel_t;
	size_t n_ts, cur_ts;
	size_t npl0, npl1;
	v3 *aei0, *aei1, *oom0, *oom1;
	double *m0, *m1;
	v3 *rdaei, *rdoom, *raei_i, *room_i;
	uint32_t* rids;
	double* rm;
	size_t n_alive;
	uint32_t* ids;            /* index -> id map (idmap inverse) */
	size_t n_ids;
	double* pm;               /* planet masses by index, as the reference keeps them in pl.m() */
} orc_interp;

static int rd(FILE* f, void* p, size_t n) { return fread(p, 1, n, f) == n ? 0 : 1; }
static double rd_f64(FILE* f, int* eof) { double x = 0; if (rd(f, &x, 8)) *eof = 1; return x; }
static uint32_t rd_u32(FILE* f, int* eof) { uint32_t x = 0; if (rd(f, &x, 4)) *eof = 1; return x; }
static float rd_f32(FILE* f, int* eof) { float x = 0; if (rd(f, &x, 4)) *eof = 1; return x; }

static size_t id_index(orc_interp* ip, uint32_t id)
{
	for (size_t k = 0; k < ip->n_ids; k++) if (ip->ids[k] == id) return k;
	ip->ids[ip->n_ids] = id;
	return ip->n_ids++;
}

static void interp_free(orc_interp* ip)
{
	if (!ip) return;
	if (ip->in) fclose(ip->in);
	free(ip->aei0); free(ip->aei1); free(ip->oom0); free(ip->oom1); free(ip->m0); free(ip->m1);
	free(ip->rdaei); free(ip->rdoom); free(ip->raei_i); free(ip->room_i); free(ip->rids); free(ip->rm);
	free(ip->ids); free(ip->pm); free(ip);
}

/* src/interp.cpp:13-91; fills the planet arrays with the first record */
static orc_interp* interp_open(const char* path, size_t cap, double user_dt, double t_0, orc_planets* pl, int* err)
{
	*err = 0;
	orc_interp* ip = (orc_interp*) calloc(1, sizeof(orc_interp));
	ip->in = fopen(path, "rb");
	if (!ip->in) { *err = 1; interp_free(ip); return NULL; }
	ip->cap = cap;
	ip->user_dt = user_dt;
	size_t n = cap;
	ip->aei0 = (v3*) calloc(n, sizeof(v3)); ip->aei1 = (v3*) calloc(n, sizeof(v3));
	ip->oom0 = (v3*) calloc(n, sizeof(v3)); ip->oom1 = (v3*) calloc(n, sizeof(v3));
	ip->m0 = (double*) calloc(n, sizeof(double)); ip->m1 = (double*) calloc(n, sizeof(double));
	ip->rdaei = (v3*) calloc(n, sizeof(v3)); ip->rdoom = (v3*) calloc(n, sizeof(v3));
	ip->raei_i = (v3*) calloc(n, sizeof(v3)); ip->room_i = (v3*) calloc(n, sizeof(v3));
	ip->rids = (uint32_t*) calloc(n, sizeof(uint32_t)); ip->rm = (double*) calloc(n, sizeof(double));
	ip->ids = (uint32_t*) calloc(n + 1, sizeof(uint32_t)); ip->pm = (double*) calloc(n, sizeof(double));
	int eof = 0;
	pl->m[0] = rd_f64(ip->in, &eof);
	fseek(ip->in, 24, SEEK_CUR);
	ip->t0 = INFINITY;
	ip->t1 = rd_f64(ip->in, &eof);
	ip->t_m1 = NAN;
	ip->npl1 = rd_u32(ip->in, &eof) + 1;
	fseek(ip->in, 20, SEEK_CUR);
	if (eof || ip->t1 > t_0) { *err = 2; interp_free(ip); return NULL; }
	ip->ids[0] = 0;
	ip->n_ids = 1;
	for (size_t i = 1; i < ip->npl1; i++)
	{
		uint32_t id = rd_u32(ip->in, &eof);
		size_t ind = id_index(ip, id);
		pl->id[ind] = id;
		ip->m1[ind] = rd_f32(ip->in, &eof);
		ip->aei1[ind].x = rd_f32(ip->in, &eof);
		ip->aei1[ind].y = rd_f32(ip->in, &eof);
		ip->aei1[ind].z = rd_f32(ip->in, &eof);
		ip->oom1[ind].x = rd_f32(ip->in, &eof);
		ip->oom1[ind].y = rd_f32(ip->in, &eof);
		ip->oom1[ind].z = rd_f32(ip->in, &eof);
		double r[3], v[3];
		orc_from_elements_M(pl->m[0] + ip->m1[ind], ip->aei1[ind].x, ip->aei1[ind].y, ip->aei1[ind].z,
			ip->oom1[ind].x, ip->oom1[ind].y, ip->oom1[ind].z, r, v);
		pl->r[i] = mk(r[0], r[1], r[2]);
		pl->v[i] = mk(v[0], v[1], v[2]);
		pl->id[i] = id;
		pl->m[i] = ip->m1[ind];
	}
	pl->r[0] = mk(0, 0, 0);
	pl->v[0] = mk(0, 0, 0);
	ip->aei1[0] = mk(0, 0, 0);
	ip->oom1[0] = mk(0, 0, 0);
	for (size_t i = 0; i < n; i++) ip->pm[i] = pl->m[i];
	return ip;
}

/* src/interp.cpp:167-293; returns nonzero at the end of the file */
static int interp_next(orc_interp* ip, orc_planets* pl)
{
	ip->t_m1 = ip->t0;
	memcpy(ip->m0, ip->m1, ip->cap * sizeof(double));
	ip->npl0 = ip->npl1;
	memcpy(ip->aei0, ip->aei1, ip->cap * sizeof(v3));
	memcpy(ip->oom0, ip->oom1, ip->cap * sizeof(v3));
	ip->t0 = ip->t1;
	ip->rel_t = 0;
	int eof = 0;
	ip->t1 = rd_f64(ip->in, &eof);
	if (eof) return 1;
	ip->npl1 = rd_u32(ip->in, &eof) + 1;
	double dt = ip->t1 - ip->t0;
	double nts = round(dt / ip->user_dt);
	ip->n_ts = nts < 1 ? 1 : (size_t) nts;
	ip->eff_dt = dt / (double) ip->n_ts;
	fseek(ip->in, 20, SEEK_CUR);
	for (size_t i = 1; i < ip->cap; i++)
	{
		ip->aei1[i] = mk(NAN, NAN, NAN);
		ip->oom1[i] = mk(NAN, NAN, NAN);
	}
	size_t k = 0;
	for (size_t i = 1; i < ip->npl1; i++)
	{
		uint32_t id = rd_u32(ip->in, &eof);
		size_t ind = id_index(ip, id);
		pl->id[ind] = id;
		ip->pm[ind] = rd_f32(ip->in, &eof);
		pl->m[ind] = ip->pm[ind];
		ip->aei1[ind].x = rd_f32(ip->in, &eof);
		ip->aei1[ind].y = rd_f32(ip->in, &eof);
		ip->aei1[ind].z = rd_f32(ip->in, &eof);
		ip->oom1[ind].x = rd_f32(ip->in, &eof);
		ip->oom1[ind].y = rd_f32(ip->in, &eof);
		ip->oom1[ind].z = rd_f32(ip->in, &eof);
		if (isnan(ip->aei0[ind].x)) continue;
		ip->rids[k] = id;
		ip->rm[k] = ip->m1[ind];
		ip->raei_i[k] = ip->aei0[ind];
		ip->room_i[k] = ip->oom0[ind];
		ip->rdaei[k] = dvs(sub(ip->aei1[ind], ip->aei0[ind]), dt);
		v3 d = sub(ip->oom1[ind], ip->oom0[ind]);
		if (d.x > ORC_PI) d.x -= 2 * ORC_PI;
		else if (d.x < -ORC_PI) d.x += 2 * ORC_PI;
		if (d.y > ORC_PI) d.y -= 2 * ORC_PI;
		else if (d.y < -ORC_PI) d.y += 2 * ORC_PI;
		d = dvs(d, dt);
		double mmfreq = 2 * ORC_PI * sqrt(1 + pl->m[ind] / pl->m[0])
			* (pow(ip->aei0[ind].x, -1.5) + pow(ip->aei1[ind].x, -1.5)) / 2;
		double cmfin = ip->oom0[ind].z + mmfreq * dt;
		cmfin = fmod(cmfin, 2 * ORC_PI);
		double corr = ip->oom1[ind].z - cmfin;
		if (corr > ORC_PI) corr -= 2 * ORC_PI;
		else if (corr < -ORC_PI) corr += 2 * ORC_PI;
		mmfreq += corr / dt;
		d.z = mmfreq;
		ip->rdoom[k] = d;
		k++;
	}
	ip->n_alive = k;
	return 0;
}

/* src/interp.cpp:93-111 */
static void interp_fill_one(orc_interp* ip, orc_planets* pl, double relative_t)
{
	for (size_t j = 0; j < ip->n_alive; j++)
	{
		v3 aei = add(ip->raei_i[j], scl(ip->rdaei[j], relative_t));
		v3 oom = add(ip->room_i[j], scl(ip->rdoom[j], relative_t));
		double gm = ip->rm[j] + pl->m[0];
		double r[3], v[3];
		orc_from_elements_M(gm, aei.x, aei.y, aei.z, oom.x, oom.y, oom.z, r, v);
		pl->r[j + 1] = mk(r[0], r[1], r[2]);
		pl->v[j + 1] = mk(v[0], v[1], v[2]);
	}
}

/* ------------------------------------------------------------------------ */
/* Executor (no encounter resolution): src/executor.cu:85-217, 226-320,     */
/* 598-764, 766-877 and WHIntegrator ctor src/wh.cpp:498-577                */
/* ------------------------------------------------------------------------ */

typedef struct
{
	int drift_kind;
	double dt, outer_r, t;
	uint32_t tbsize;
	int interp_mode;
	orc_planets* pl;          /* live planet state (one block ahead of the particles) */
	orc_interp* ip;
	double cur_dt;
	size_t cur_tbsize;
	/* the planet block the next loop integrates with */
	double *r_log, *h0_log, *blk_m, *blk_rh;
	uint32_t* blk_id;
	uint32_t blk_npl, blk_len;
	/* planet snapshot at the particles' time */
	size_t snap_n;
	double *snap_m, *snap_r, *snap_v;
	uint32_t* snap_id;
	/* particles (kept in device order) */
	size_t n, n_alive;
	double *r, *v, *a, *deathtime;
	uint32_t *id, *dti;
	uint16_t* flags;
	char err[256];
} orc_exec;

static void snapshot(orc_exec* e)
{
	orc_planets* p = e->pl;
	e->snap_n = e->interp_mode ? e->ip->n_alive + 1 : p->n;
	for (size_t i = 0; i < e->snap_n; i++)
	{
		e->snap_m[i] = p->m[i];
		st(e->snap_r, i, p->r[i]);
		st(e->snap_v, i, p->v[i]);
		e->snap_id[i] = p->id[i];
	}
}

static int update_planets(orc_exec* e)
{
	orc_planets* p = e->pl;
	size_t npl_live = e->interp_mode ? e->ip->n_alive + 1 : p->n;
	/* rh uses the live planets with the reference's full count pl.n() */
	size_t keep = p->n;
	recalculate_rh(p);
	p->n = keep;
	if (e->interp_mode)
	{
		orc_interp* ip = e->ip;
		if (ip->cur_ts == ip->n_ts)
		{
			if (interp_next(ip, p)) { snprintf(e->err, sizeof e->err, "EOS reached for lookup file."); return -7; }
			ip->cur_ts = 0;
			e->t = ip->t0;
		}
		e->cur_dt = ip->eff_dt;
		size_t left = ip->n_ts - ip->cur_ts;
		e->cur_tbsize = e->tbsize < left ? e->tbsize : left;
		/* src/interp.cpp:113-165 */
		npl_live = ip->n_alive + 1;
		double relt = ip->rel_t + e->cur_dt;
		for (size_t j = 0; j < ip->n_alive; j++)
		{
			p->id[j + 1] = ip->rids[j];
			p->m[j + 1] = ip->rm[j];
		}
		for (size_t i = 0; i < e->cur_tbsize; i++)
		{
			if (relt > ip->t1 - ip->t0 + 1e-8)
			{
				snprintf(e->err, sizeof e->err, "interpolation ran too long, timechunk exceeded lookup boundary");
				return -8;
			}
			p->r[0] = mk(0, 0, 0);
			p->v[0] = mk(0, 0, 0);
			interp_fill_one(ip, p, relt);
			for (size_t j = 0; j < ip->n_alive; j++) st(e->r_log, i * ip->n_alive + j, p->r[j + 1]);
			relt += e->cur_dt;
		}
		ip->rel_t += (double) e->cur_tbsize * e->cur_dt;
		ip->cur_ts += e->cur_tbsize;
		/* src/wh.cpp:993-1025 */
		for (size_t idx = 0; idx < e->cur_tbsize; idx++)
		{
			v3 h0 = mk(0, 0, 0), a_common = mk(0, 0, 0);
			for (size_t i = 1; i < npl_live; i++)
			{
				v3 r = ld(e->r_log, idx * (npl_live - 1) + i - 1);
				double r2 = lensq(r);
				double inv_r3 = 1. / (sqrt(r2) * r2);
				if (i == 1) h0 = scl(scl(mk(-r.x, -r.y, -r.z), p->m[1]), inv_r3);
				if (i > 1)
				{
					double mfac = p->m[i] * inv_r3;
					a_common = sub(a_common, scl(r, mfac));
				}
			}
			h0 = add(h0, a_common);
			st(e->h0_log, idx, h0);
		}
	}
	else
	{
		e->cur_dt = e->dt;
		e->cur_tbsize = e->tbsize;
		for (size_t i = 0; i < e->cur_tbsize; i++)
		{
			v3 h0;
			int err = step_planets(p, e->cur_dt, e->r_log + 3 * i * (p->n - 1), &h0);
			if (err)
			{
				snprintf(e->err, sizeof e->err, err == 1 ? "unbound orbit of planet" : "Unconverging kepler");
				return -8;
			}
			st(e->h0_log, i, h0);
		}
	}
	e->blk_npl = (uint32_t) npl_live;
	e->blk_len = (uint32_t) e->cur_tbsize;
	for (size_t i = 0; i < npl_live; i++)
	{
		e->blk_m[i] = p->m[i];
		e->blk_id[i] = p->id[i];
		e->blk_rh[i] = p->rh[i];
	}
	return 0;
}

void orc_exec_free(orc_exec* e);

/* Stable partition of rows [begin, begin+len): rows with (flags & mask) == 0
 * first; returns their count. */
static size_t stable_partition_rows(orc_exec* e, size_t begin, size_t len, uint16_t mask)
{
	size_t n = len;
	double* tr = (double*) malloc(24 * n + 8);
	double* tv = (double*) malloc(24 * n + 8);
	double* ta = (double*) malloc(24 * n + 8);
	double* td = (double*) malloc(8 * n + 8);
	uint32_t* tid = (uint32_t*) malloc(4 * n + 4);
	uint32_t* tdti = (uint32_t*) malloc(4 * n + 4);
	uint16_t* tf = (uint16_t*) malloc(2 * n + 2);
	size_t w = 0, keep = 0;
	for (int pass = 0; pass < 2; pass++)
	{
		for (size_t k = 0; k < n; k++)
		{
			size_t i = begin + k;
			int first = (e->flags[i] & mask) == 0;
			if (first != (pass == 0)) continue;
			keep += first;
			memcpy(tr + 3 * w, e->r + 3 * i, 24);
			memcpy(tv + 3 * w, e->v + 3 * i, 24);
			memcpy(ta + 3 * w, e->a + 3 * i, 24);
			td[w] = e->deathtime[i];
			tid[w] = e->id[i];
			tdti[w] = e->dti[i];
			tf[w] = e->flags[i];
			w++;
		}
	}
	memcpy(e->r + 3 * begin, tr, 24 * n); memcpy(e->v + 3 * begin, tv, 24 * n); memcpy(e->a + 3 * begin, ta, 24 * n);
	memcpy(e->deathtime + begin, td, 8 * n); memcpy(e->id + begin, tid, 4 * n); memcpy(e->dti + begin, tdti, 4 * n);
	memcpy(e->flags + begin, tf, 2 * n);
	free(tr); free(tv); free(ta); free(td); free(tid); free(tdti); free(tf);
	return keep;
}


/* Creates a run from arrays.  Planet vectors are [npl][3] in any inertial
 * frame (converted to heliocentric as Executor::init does).  interp_path may
 * be NULL for the direct planet integrator. */
orc_exec* orc_exec_new(int drift_kind, int ref_quirks, double t0, double dt, uint32_t tbsize, double outer_r, double cull_r,
	double esf, const char* interp_path, uint32_t interp_maxpl,
	size_t npl, const double* pm, const double* pr, const double* pv, const uint32_t* pid,
	size_t n, const double* r, const double* v, const uint32_t* id, const uint16_t* flags)
{
	orc_exec* e = (orc_exec*) calloc(1, sizeof(orc_exec));
	e->drift_kind = drift_kind;
	e->t = t0;
	e->dt = dt;
	e->tbsize = tbsize;
	e->outer_r = outer_r;
	e->interp_mode = interp_path != NULL;
	size_t cap = e->interp_mode ? interp_maxpl : npl;
	e->pl = planets_new(cap);
	orc_planets* p = e->pl;
	p->cull_radius = cull_r;
	p->esf = esf;
	v3 r0 = mk(0, 0, 0), v0 = mk(0, 0, 0);
	if (!e->interp_mode)
	{
		r0 = ld(pr, 0);
		v0 = ld(pv, 0);
		for (size_t i = 0; i < npl; i++)
		{
			p->m[i] = pm[i];
			p->r[i] = sub(ld(pr, i), r0);
			p->v[i] = sub(ld(pv, i), v0);
			p->id[i] = pid[i];
		}
	}
	else
	{
		/* the state file's planets only fix the frame */
		if (npl > 0) { r0 = ld(pr, 0); v0 = ld(pv, 0); }
	}
	e->n = n;
	e->r = (double*) calloc(3 * n + 3, sizeof(double));
	e->v = (double*) calloc(3 * n + 3, sizeof(double));
	e->a = (double*) calloc(3 * n + 3, sizeof(double));
	e->deathtime = (double*) calloc(n + 1, sizeof(double));
	e->id = (uint32_t*) calloc(n + 1, sizeof(uint32_t));
	e->dti = (uint32_t*) calloc(n + 1, sizeof(uint32_t));
	e->flags = (uint16_t*) calloc(n + 1, sizeof(uint16_t));
	for (size_t i = 0; i < n; i++)
	{
		st(e->r, i, sub(ld(r, i), r0));
		st(e->v, i, sub(ld(v, i), v0));
		e->id[i] = id[i];
		e->flags[i] = flags ? flags[i] : 0;
	}
	size_t maxpl = cap;
	e->r_log = (double*) calloc(3 * (size_t) tbsize * maxpl + 3, sizeof(double));
	e->h0_log = (double*) calloc(3 * (size_t) tbsize + 3, sizeof(double));
	e->blk_m = (double*) calloc(maxpl, sizeof(double));
	e->blk_rh = (double*) calloc(maxpl, sizeof(double));
	e->blk_id = (uint32_t*) calloc(maxpl, sizeof(uint32_t));
	e->snap_m = (double*) calloc(maxpl, sizeof(double));
	e->snap_r = (double*) calloc(3 * maxpl, sizeof(double));
	e->snap_v = (double*) calloc(3 * maxpl, sizeof(double));
	e->snap_id = (uint32_t*) calloc(maxpl, sizeof(uint32_t));

	if (e->interp_mode)
	{
		int err;
		e->ip = interp_open(interp_path, interp_maxpl, dt, t0, p, &err);
		if (!e->ip) { orc_exec_free(e); return NULL; }
		orc_interp* ip = e->ip;
		while (ip->t1 <= e->t)
		{
			if (interp_next(ip, p)) { orc_exec_free(e); return NULL; }
		}
		ip->cur_ts = 0;
		double nts = round((ip->t1 - e->t) / dt);
		ip->n_ts = nts < 1 ? 1 : (size_t) nts;
		ip->eff_dt = (ip->t1 - e->t) / (double) ip->n_ts;
		ip->rel_t = e->t - ip->t0;
		interp_fill_one(ip, p, ip->rel_t);
	}
	/* WHIntegrator ctor, src/wh.cpp:498-577 */
	size_t nl = e->interp_mode ? e->ip->n_alive + 1 : p->n;
	p->eta[0] = p->m[0];
	for (size_t i = 1; i < p->n; i++) p->eta[i] = p->eta[i - 1] + p->m[i];
	recalculate_rh(p);
	helio_to_jacobi_r(p);
	helio_to_jacobi_v(p);
	v3 h0;
	size_t keep = p->n;
	p->n = nl;
	helio_acc_planets(p, &h0);
	p->n = keep;
	/* helio_acc_particle<old=true> at index 0, src/wh.cpp:611-657 */
	for (size_t k = 0; k < n; k++)
	{
		v3 acc = h0;
		v3 rk = ld(e->r, k);
		for (size_t j = 1; j < nl; j++)
		{
			v3 dr = sub(rk, p->r[j]);
			double rji2 = lensq(dr);
			double irij3 = 1. / (rji2 * sqrt(rji2));
			double fac = p->m[j] * irij3;
			acc = sub(acc, scl(dr, fac));
			if (rji2 < p->rh[j] * p->rh[j])
			{
				e->deathtime[k] = 0;
				e->flags[k] = (uint16_t) ((j << 8) | 0x0001);
			}
		}
		double rji2 = lensq(rk);
		/* the reference passes time 0 here, not Initial-Time (src/wh.cpp:543) */
		if (rji2 < p->rh[0] * p->rh[0]) { e->deathtime[k] = 0; e->flags[k] = 0x0001; }
		if (rji2 > outer_r * outer_r) { e->deathtime[k] = 0; e->flags[k] = 0x0002; }
		st(e->a, k, acc);
	}
	/* src/executor.cu:181-187: stable partitions, unflagged first, then the
	 * encounter particles among the rest.  With ref_quirks the accelerations
	 * stay in their pre-partition order, as the reference uploads them
	 * (integrator.particle_a is never gathered) -- a reference defect that
	 * only shows when a particle is flagged at start. */
	double* a_keep = NULL;
	if (ref_quirks)
	{
		a_keep = (double*) malloc(24 * n + 8);
		memcpy(a_keep, e->a, 24 * n);
	}
	size_t na = stable_partition_rows(e, 0, n, 0xFFFF);
	na += stable_partition_rows(e, na, n - na, 0x00FE);
	e->n_alive = na;
	if (a_keep)
	{
		memcpy(e->a, a_keep, 24 * n);
		free(a_keep);
	}
	snapshot(e);
	if (update_planets(e)) { orc_exec_free(e); return NULL; }
	return e;
}

void orc_exec_free(orc_exec* e)
{
	if (!e) return;
	planets_free(e->pl);
	interp_free(e->ip);
	free(e->r); free(e->v); free(e->a); free(e->deathtime); free(e->id); free(e->dti); free(e->flags);
	free(e->r_log); free(e->h0_log); free(e->blk_m); free(e->blk_rh); free(e->blk_id);
	free(e->snap_m); free(e->snap_r); free(e->snap_v); free(e->snap_id);
	free(e);
}

/* One block of Executor::loop without encounter resolution.  Returns 0, or
 * a negative code with the message in orc_exec_error. */
int orc_exec_loop(orc_exec* e)
{
	size_t prev_alive = e->n_alive;
	size_t presort = 0;
	if (e->n_alive > 0)
	{
		orc_block(e->drift_kind, e->n_alive, e->r, e->v, e->a, e->flags, e->dti, e->blk_len, e->blk_npl,
			e->h0_log, e->r_log, e->blk_m, e->blk_id, e->blk_rh, e->outer_r, e->cur_dt, e->blk_m[0]);
		for (size_t i = 0; i < e->n_alive; i++)
		{
			uint16_t f = e->flags[i];
			if ((f & 0x01) == 0x01) e->flags[i] = (uint16_t) ((f & 0xFF00) | 0x80);
		}
		presort = stable_partition_rows(e, 0, e->n_alive, 0xFFFF);
	}
	snapshot(e);
	e->t += e->cur_dt * (double) e->cur_tbsize;
	int err = update_planets(e);
	if (prev_alive > 0)
	{
		e->n_alive = presort;
		for (size_t i = presort; i < prev_alive; i++) e->deathtime[i] = (float) e->t;
	}
	return err;
}

const char* orc_exec_error(orc_exec* e) { return e->err; }

void orc_exec_counts(orc_exec* e, size_t* n, size_t* n_alive, double* t, uint32_t* npl, uint32_t* len)
{
	*n = e->n;
	*n_alive = e->n_alive;
	*t = e->t;
	*npl = e->blk_npl;
	*len = e->blk_len;
}

void orc_exec_particles(orc_exec* e, double* r, double* v, double* a, uint32_t* id, uint16_t* flags, uint32_t* dti, double* deathtime)
{
	memcpy(r, e->r, 24 * e->n);
	memcpy(v, e->v, 24 * e->n);
	memcpy(a, e->a, 24 * e->n);
	memcpy(id, e->id, 4 * e->n);
	memcpy(flags, e->flags, 2 * e->n);
	memcpy(dti, e->dti, 4 * e->n);
	memcpy(deathtime, e->deathtime, 8 * e->n);
}

void orc_exec_planet_block(orc_exec* e, double* r_log, double* h0_log, double* m, uint32_t* id, double* rh)
{
	memcpy(r_log, e->r_log, 24 * (size_t) e->blk_len * (e->blk_npl - 1));
	memcpy(h0_log, e->h0_log, 24 * (size_t) e->blk_len);
	memcpy(m, e->blk_m, 8 * e->blk_npl);
	memcpy(id, e->blk_id, 4 * e->blk_npl);
	memcpy(rh, e->blk_rh, 8 * e->blk_npl);
}

void orc_exec_planets(orc_exec* e, size_t* n, double* m, double* r, double* v, uint32_t* id)
{
	*n = e->snap_n;
	memcpy(m, e->snap_m, 8 * e->snap_n);
	memcpy(r, e->snap_r, 24 * e->snap_n);
	memcpy(v, e->snap_v, 24 * e->snap_n);
	memcpy(id, e->snap_id, 4 * e->snap_n);
}

/* Planet-only integration to produce the history blocks for a fixture:
 * runs nsteps WH steps of the planets from heliocentric state and writes
 * [nsteps][npl-1][3] positions and [nsteps][npl][3] velocities after each
 * step (src/wh.cpp:1027-1067). */
int orc_planet_steps(size_t npl, const double* m, double* r, double* v, double dt, size_t nsteps, double* r_out, double* v_out, double* h0_out)
{
	orc_planets* p = planets_new(npl);
	for (size_t i = 0; i < npl; i++)
	{
		p->m[i] = m[i];
		p->r[i] = sub(ld(r, i), ld(r, 0));
		p->v[i] = sub(ld(v, i), ld(v, 0));
	}
	p->eta[0] = p->m[0];
	for (size_t i = 1; i < npl; i++) p->eta[i] = p->eta[i - 1] + p->m[i];
	helio_to_jacobi_r(p);
	helio_to_jacobi_v(p);
	v3 h0;
	helio_acc_planets(p, &h0);
	int err = 0;
	for (size_t s = 0; s < nsteps && !err; s++)
	{
		err = step_planets(p, dt, r_out + 3 * s * (npl - 1), &h0);
		if (h0_out) st(h0_out, s, h0);
		if (v_out) for (size_t i = 0; i < npl; i++) st(v_out, s * npl + i, p->v[i]);
	}
	for (size_t i = 0; i < npl; i++) { st(r, i, p->r[i]); st(v, i, p->v[i]); }
	planets_free(p);
	return err;
}

/* Time step of the block the next orc_exec_loop integrates. */
double orc_exec_dt(orc_exec* e) { return e->cur_dt; }
