"""Edge cases: many planets (the generic planet loop past the specialised
counts), a single particle, every particle flagged at start, ensembles with
empty and one-particle systems and with more planets than the device planet
integrator takes."""
import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import glisser_gb300 as G  # noqa: E402
from glisser_gb300 import synth  # noqa: E402

CFG = ("Time-Step 180\nTime-Block-Size %d\nFinal-Time 1e30\nCull-Radius 0.5\nOuter-Limit 300\n"
       "Input-File unused\nOutput-Folder unused\n")


@pytest.fixture(scope="module", autouse=True)
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    G.build()
    G.lib()


def planets(k, seed=0):
    """Sun + k small planets on near-circular orbits from 5 to 45 au."""
    rng = np.random.default_rng(seed)
    mu = synth.GM_SUN_AU_DAY
    m = np.concatenate([[mu], rng.uniform(1e-7, 5e-6, k) * mu])
    pr, pv = [np.zeros(3)], [np.zeros(3)]
    for j, a in enumerate(np.linspace(5, 45, k)):
        el = np.array([[a, rng.uniform(0, 0.05), rng.uniform(0, 0.03), rng.uniform(0, 6.28), rng.uniform(0, 6.28),
                        rng.uniform(0, 6.28)]])
        r, v = G.elements_to_cartesian(m[0] + m[j + 1], el)
        pr.append(r[0]); pv.append(v[0])
    return m, np.array(pr), np.array(pv)


def by_id(p):
    o = np.argsort(p["id"])
    return {k: np.asarray(v)[o] for k, v in p.items()}


@pytest.mark.parametrize("k", [9, 12])
def test_many_planets_match_oracle(k):
    m, pr, pv = planets(k, seed=k)
    el = synth.particle_elements(np.random.default_rng(5), 300, (20, 50), (0, 0.2), 10.0)
    r, v = G.elements_to_cartesian(m[0], el)
    sim = G.Simulation(CFG % 64)
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v)
    sim.init()
    ex = O.Exec(m, pr, pv, np.arange(len(m)), r, v, np.arange(len(r)), dt=180.0, tbsize=64, outer_r=300.0,
                cull_r=0.5)
    for b in range(4):
        sim.loop()
        ex.loop()
        got, want = by_id(sim.particles()), by_id(ex.particles())
        assert np.array_equal(got["flags"], want["flags"]), b
    live = want["flags"] == 0
    err = np.linalg.norm(got["r"] - want["r"], axis=1) / np.linalg.norm(want["r"], axis=1)
    assert err[live].max() < 1e-10


def test_single_particle_and_all_flagged_start():
    m, pr, pv, r, v = synth.cartesian_state("plain-neptune", 1, seed=2)
    sim = G.Simulation(CFG % 32)
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v)
    sim.init()
    sim.loop()
    assert sim.counts()["n_alive"] == 1 and sim.stats()["particle_steps"] == 32
    # every particle outside the outer limit: flagged at init, nothing integrates
    far = np.tile([[400.0, 0.0, 0.0]], (5, 1))
    vel = np.tile([[0.0, 1e-4, 0.0]], (5, 1))
    sim2 = G.Simulation(CFG % 32)
    sim2.set_planets(m, pr, pv)
    sim2.set_particles(far, vel)
    sim2.init()
    sim2.loop()
    c = sim2.counts()
    assert c["n_alive"] == 0
    assert np.all(sim2.particles()["flags"] == 0x02)


def test_ensemble_with_empty_and_tiny_systems():
    syst = []
    for s, n in enumerate([0, 1, 700, 0, 33]):
        m, pel, el = synth.ensemble_workload(1, seed=40 + s, counts=np.array([max(n, 1)]))[0]
        pr, pv = [np.zeros(3)], [np.zeros(3)]
        for k in range(4):
            a, b = G.elements_to_cartesian(m[0] + m[k + 1], pel[k:k + 1])
            pr.append(a[0]); pv.append(b[0])
        r, v = G.elements_to_cartesian(m[0], el)
        syst.append((m, np.array(pr), np.array(pv), r[:n], v[:n]))
    ens = G.Ensemble(CFG % 64, len(syst))
    for s, (m, pr, pv, r, v) in enumerate(syst):
        ens.set_system(s, m, pr, pv, r, v)
    ens.init()
    for _ in range(3):
        ens.step()
    for s, (m, pr, pv, r, v) in enumerate(syst):
        c = ens.counts(s)
        assert c["n"] == len(r)
        if len(r) == 0:
            continue
        sim = G.Simulation(CFG % 64)
        sim.set_planets(m, pr, pv)
        sim.set_particles(r, v)
        sim.init()
        for _ in range(3):
            sim.loop()
        want = by_id(sim.particles())
        got = ens.particles(s)
        assert np.array_equal(got["flags"], want["flags"])
        err = np.linalg.norm(got["r"] - want["r"], axis=1) / np.linalg.norm(want["r"], axis=1)
        assert err.max() < 1e-10


def test_ensemble_beyond_device_planet_limit_uses_host_planets():
    m, pr, pv = planets(40, seed=3)                          # 41 bodies > 32
    el = synth.particle_elements(np.random.default_rng(6), 64, (20, 50), (0, 0.1), 5.0)
    r, v = G.elements_to_cartesian(m[0], el)
    ens = G.Ensemble(CFG % 32, 2)
    ens.set_system(0, m, pr, pv, r, v)
    ens.set_system(1, m, pr, pv, r[:10], v[:10])
    ens.init()
    ens.step()
    l0 = ens.stats()["launches"]
    ens.step()
    assert ens.stats()["launches"] - l0 == 1               # the graph only: planets on the host
    sim = G.Simulation(CFG % 32)
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v)
    sim.init()
    sim.loop(); sim.loop()
    want = by_id(sim.particles())
    got = ens.particles(0)
    err = np.linalg.norm(got["r"] - want["r"], axis=1) / np.linalg.norm(want["r"], axis=1)
    assert err.max() < 1e-12


@pytest.mark.parametrize("units", ["si", "tiny"])
def test_units_do_not_change_the_orbits(units):
    """The same system in SI units (metres, seconds: |dr|^2 ~ 1e24, past the
    float-float pull's range, so its FP64 branch runs) and in units that make
    every length 1e-6 of an au: after 512 steps the positions, rescaled, match
    the au/day run to 1e-12 with the same flags, and the au/day run matches
    the oracle."""
    m, pr, pv = planets(4, seed=3)
    el = synth.particle_elements(np.random.default_rng(8), 256, (20, 50), (0, 0.2), 10.0)
    r, v = G.elements_to_cartesian(m[0], el)
    Lu, Tu = (1.495978707e11, 86400.0) if units == "si" else (1e-6, 1.0)
    runs = []
    for L, Tt in ((1.0, 1.0), (Lu, Tu)):
        cfg = ("Time-Step %r\nTime-Block-Size 128\nFinal-Time 1e30\nCull-Radius %r\nOuter-Limit %r\n"
               "Input-File unused\nOutput-Folder unused\n" % (180.0 * Tt, 0.5 * L, 300.0 * L))
        sim = G.Simulation(cfg)
        sim.set_planets(m * L ** 3 / Tt ** 2, pr * L, pv * L / Tt)
        sim.set_particles(r * L, v * L / Tt)
        sim.init()
        for _ in range(4):
            sim.loop()
        p = by_id(sim.particles())
        runs.append((p["r"] / L, p["flags"]))
    (ra, fa), (rb, fb) = runs
    assert np.array_equal(fa, fb)
    live = fa == 0
    err = np.linalg.norm(ra - rb, axis=1) / np.linalg.norm(ra, axis=1)
    assert err[live].max() < 1e-12, err[live].max()
    ex = O.Exec(m, pr, pv, np.arange(len(m)), r, v, np.arange(len(r)), dt=180.0, tbsize=128, outer_r=300.0,
                cull_r=0.5)
    for _ in range(4):
        ex.loop()
    want = by_id(ex.particles())
    assert np.array_equal(want["flags"], fa)
    err = np.linalg.norm(ra - want["r"], axis=1) / np.linalg.norm(want["r"], axis=1)
    assert err[live].max() < 1e-10
