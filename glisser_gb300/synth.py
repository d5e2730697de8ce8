"""Seeded synthetic workloads (orbital elements; angles in radians): the five
benchmark workloads, named for what they are -- plain-neptune, plain-giants,
scattered-disk, ensembles, history-encounters -- and close-eccentric, the
regime of the scattered disk's pericentre passages on its own (every drift a
sizeable part of the local dynamical time, tau^2 = dt^2 mu / r^3 > 0.01, where
the series starter does not apply and the learned starter runs its network).

The reference ships no particle state for its examples (the 200,000-particle
resonance state is not distributed), so every workload here is generated:
numpy's default generator seeded per workload draws the elements and
`from_elements_M` (src/convert.cpp:257-275, restated in the library) turns
them into heliocentric Cartesian states.
"""
import numpy as np

DEG = np.pi / 180.0
GM_SUN_AU_DAY = 2.959122e-4            # G*Msun in au^3/day^2 (G = 1 units)
GM_SUN_AU_YR = 4 * np.pi ** 2          # G*Msun in au^3/yr^2

GIANT_MASSES = np.array([9.55e-4, 2.86e-4, 4.37e-5, 5.15e-5])   # in Msun
GIANT_A = np.array([5.2, 9.55, 19.2, 30.1])
NEPTUNE_MASS = 5.15e-5


def _angles(rng, n):
    return rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n)


def particle_elements(rng, n, a_range, e_range, i_max_deg, log_a=False):
    """Elements [n, 6] = a, e, i, capom, om, M with uniform angles."""
    if log_a:
        a = np.exp(rng.uniform(np.log(a_range[0]), np.log(a_range[1]), n))
    else:
        a = rng.uniform(a_range[0], a_range[1], n)
    e = rng.uniform(e_range[0], e_range[1], n)
    inc = rng.uniform(0, i_max_deg * DEG, n)
    O, o, M = _angles(rng, n)
    return np.stack([a, e, inc, O, o, M], axis=1)


def neptune_planets(gm_sun=GM_SUN_AU_DAY, a=30.0):
    """Sun + one Neptune-mass planet on a circular, planar orbit (plain-neptune,
    scattered-disk, history-encounters).
    Returns (masses [2], elements [1, 6])."""
    m = np.array([gm_sun, NEPTUNE_MASS * gm_sun])
    el = np.array([[a, 0.0, 0.0, 0.0, 0.0, 0.0]])
    return m, el


def giant_planets(rng, gm_sun=GM_SUN_AU_DAY, mass_scale=None, a_scale=None):
    """Sun + four giants with e~U(0,0.05), i~U(0,2 deg) (plain-giants, ensembles)."""
    ms = GIANT_MASSES * (mass_scale if mass_scale is not None else 1.0)
    a = GIANT_A * (a_scale if a_scale is not None else 1.0)
    e = rng.uniform(0, 0.05, 4)
    inc = rng.uniform(0, 2 * DEG, 4)
    O, o, M = _angles(rng, 4)
    m = np.concatenate([[gm_sun], ms * gm_sun])
    return m, np.stack([a, e, inc, O, o, M], axis=1)


WORKLOADS = {
    "plain-neptune": dict(n=2000, dt=180.0, steps=10000, tbsize=128, cull=0.5, outer=300.0,
                          planets="neptune", a=(40, 50), e=(0, 0.1), i=5.0),
    "plain-giants": dict(n=1_000_000, dt=180.0, steps=200_000, tbsize=2048, cull=0.5, outer=300.0,
                         planets="giants", a=(53, 57), e=(0, 0.3), i=10.0),
    "scattered-disk": dict(n=1_000_000, dt=180.0, steps=50_000, tbsize=512, cull=0.5, outer=1e5,
                           planets="neptune", a=(30, 1000), e=(0, 0.95), i=40.0, log_a=True),
    "ensembles": dict(systems=256, median=20000, clip=(1000, 200000), dt=180.0, steps=10000, tbsize=1024,
                      cull=0.5, outer=300.0, planets="giants", a=(40, 50), e=(0, 0.1), i=5.0),
    "history-encounters": dict(n=2_000_000, dt=0.2, steps=50_000, tbsize=100, cull=0.5, outer=300.0,
                               planets="neptune-yr", a=(20, 40), e=(0, 0.3), i=10.0, esf=3.0, hist_every=100),
    # r = a (1 +- e) within 1.0 .. 9.6 au: tau^2 >= 0.0108 at dt = 180 d
    "close-eccentric": dict(n=1_000_000, dt=180.0, steps=10_000, tbsize=512, cull=0.5, outer=1e5,
                            planets="neptune", a=(2.5, 6.0), e=(0.1, 0.6), i=20.0),
}


def workload(name, n=None, seed=0):
    """Returns dict(pl_m [npl], pl_el [npl-1, 6], el [n, 6], name, **parameters)
    for the named workload."""
    c = dict(WORKLOADS[name], name=name)
    rng = np.random.default_rng(seed)
    if c["planets"] == "neptune":
        m, pel = neptune_planets()
    elif c["planets"] == "neptune-yr":
        m, pel = neptune_planets(GM_SUN_AU_YR)
    else:
        m, pel = giant_planets(rng)
    n = c.get("n", 0) if n is None else n
    el = particle_elements(rng, n, c["a"], c["e"], c["i"], c.get("log_a", False))
    c.update(pl_m=m, pl_el=pel, el=el, n=n)
    return c


def ensemble_counts(systems=256, median=20000, clip=(1000, 200000), sigma=0.6, seed=0):
    """Lognormal particle counts per system (ensembles; sigma 0.6 gives ~6e6
    particles over 256 systems)."""
    rng = np.random.default_rng(seed)
    c = np.exp(rng.normal(np.log(median), sigma, systems))
    return np.clip(np.round(c), clip[0], clip[1]).astype(np.int64)


def ensemble_workload(systems=256, seed=0, fraction=1.0, counts=None):
    """Ensembles: per system (planet masses [5], planet elements [4, 6],
    particle elements [n, 6]); giant masses x U(0.9, 1.1) and semi-major axes
    x U(0.95, 1.05) per system, particles with the plain-neptune distributions.
    Sub-seed per system = seed + system index.  `fraction` keeps that share of
    every system's particles (at least one)."""
    if counts is None:
        counts = ensemble_counts(systems, seed=seed)
    out = []
    for s in range(systems):
        rng = np.random.default_rng(seed + s)
        m, pel = giant_planets(rng, mass_scale=rng.uniform(0.9, 1.1, 4), a_scale=rng.uniform(0.95, 1.05, 4))
        n = max(1, int(round(counts[s] * fraction)))
        el = particle_elements(rng, n, (40, 50), (0, 0.1), 5.0)
        out.append((m, pel, el))
    return out


def cartesian_state(name, n, seed, planet_seed=0):
    """Planets (m [npl], r [npl, 3], v [npl, 3]; Sun at the origin) of the
    named workload drawn with `planet_seed`, and n particles (r, v [n, 3])
    drawn with `seed`, heliocentric."""
    from . import elements_to_cartesian
    w = workload(name, n=0, seed=planet_seed)
    el = workload(name, n=n, seed=seed)["el"]
    m = w["pl_m"]
    pr, pv = [np.zeros(3)], [np.zeros(3)]
    for k in range(len(m) - 1):
        a, b = elements_to_cartesian(m[0] + m[k + 1], w["pl_el"][k:k + 1])
        pr.append(a[0])
        pv.append(b[0])
    r, v = elements_to_cartesian(m[0], el)
    return m, np.array(pr), np.array(pv), r, v
