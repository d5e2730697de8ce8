"""The batched (ensemble) kernel, the learned starter and the planetary-history
workload against the FP64 oracle directly.

Every result is compared with the oracle's block loop (oracle/glisser_oracle.c,
the reference's src/executor.cu loop over its WH planet integrator and the
universal-variable drift of src/wh.cpp:131-420), not with another run of this
library: flags, deathtime indices, deathtimes, ids and alive counts exactly,
positions within 1e-10 relative per 1e3 steps (for the Neptune crossers, whose
passages just outside three Hill radii are chaotic, 99 % of the survivors
within that bound and every one within 1e-8).

  * Ensembles shaped as the 256-system benchmark workload (giant masses x
    U(0.9, 1.1), semi-major axes x U(0.95, 1.05), uneven particle counts from
    1e3 to 1.2e4, one system of Neptune crossers that get culled or flagged
    within three Hill radii), run with the series, classic and learned
    starters through glisser_ensemble_*.
  * The learned starter where its network runs: an ensemble at dt = 20 d with
    a system of inner eccentric particles (drifts with tau^2 >= 0.01), and the
    network trained on that system's own logged plain solves.
  * The planetary-history workload (history written by the library's planet
    integrator, evaluated on the device, 3 Hill-radius encounter flags) with
    the learned starter.

The oracle runs one system per thread (ctypes releases the GIL).
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import glisser_gb300 as G  # noqa: E402
from glisser_gb300 import learned as L  # noqa: E402
from glisser_gb300 import synth  # noqa: E402

POS_TOL = 1e-10
# Encounter-RH-Factor 3, as the history workload: a particle that comes
# within three Hill radii of a planet is flagged and removed, so the survivors
# compared are those without close approaches (whose orbits magnify rounding
# differences without bound)
ESF = 3.0
CFG = ("Time-Step %r\nTime-Block-Size %d\nFinal-Time 1e30\nCull-Radius 0.5\nOuter-Limit %r\n"
       "Encounter-RH-Factor 3\nInput-File x\nOutput-Folder x\n")


@pytest.fixture(scope="module", autouse=True)
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    G.build()
    G.lib()
    O.build()


def cartesian(m, pel, el):
    pr, pv = [np.zeros(3)], [np.zeros(3)]
    for k in range(len(m) - 1):
        a, b = G.elements_to_cartesian(m[0] + m[k + 1], pel[k:k + 1])
        pr.append(a[0])
        pv.append(b[0])
    r, v = G.elements_to_cartesian(m[0], el)
    return m, np.array(pr), np.array(pv), r, v


def benchmark_shaped_systems(seed=41):
    """Six systems of the ensemble workload's kind with uneven counts; system
    2 holds eccentric Neptune crossers (a 20-45 au, e 0.3-0.8) so that the
    outer limit (60 au) and the cull radius remove particles."""
    counts = np.array([1000, 12000, 2500, 6000, 1500, 3000])
    out = []
    for s, (m, pel, el) in enumerate(synth.ensemble_workload(len(counts), seed=seed, counts=counts)):
        if s == 2:
            el = synth.particle_elements(np.random.default_rng(seed + 100), counts[s], (20, 45), (0.3, 0.8), 10.0)
        out.append(cartesian(m, pel, el))
    return out


INNER_DT = 20.0


def inner_system(n, seed):
    """Giants of the ensemble workload and particles well inside Jupiter on
    eccentric orbits (a 1.5-2.5 au, e 0.05-0.3): at dt = 20 d (34-72 steps
    per orbit) the drifts inside 2.3 au have tau^2 = dt^2 mu / r^3 >= 0.01,
    where the learned starter runs its network."""
    rng = np.random.default_rng(seed)
    m, pel = synth.giant_planets(rng, mass_scale=rng.uniform(0.9, 1.1, 4), a_scale=rng.uniform(0.95, 1.05, 4))
    el = synth.particle_elements(rng, n, (1.5, 2.5), (0.05, 0.3), 10.0)
    return cartesian(m, pel, el)


def oracle_runs(systems, dt, T, blocks, outer):
    """Each system through the oracle's block loop (universal-variable drift);
    returns per system the particles after every block and the alive counts."""
    def run(sysm):
        m, pr, pv, r, v = sysm
        ex = O.Exec(m, pr, pv, np.arange(len(m)), r, v, np.arange(len(r)), dt=dt, tbsize=T, outer_r=outer,
                    cull_r=0.5, esf=ESF, drift="uv")
        out = []
        for _ in range(blocks):
            ex.loop()
            p = ex.particles()
            o = np.argsort(p["id"])
            out.append(({k: p[k][o] for k in ("r", "v", "id", "flags", "dti", "deathtime")}, ex.counts()["n_alive"]))
        return out

    with ThreadPoolExecutor(max_workers=min(len(systems), os.cpu_count() or 1)) as pool:
        return list(pool.map(run, systems))


def run_ensemble(systems, dt, T, blocks, outer, starter, mlp_path=None, cta=64, ppt=1):
    ens = G.Ensemble(CFG % (dt, T, outer), len(systems))
    for s, (m, pr, pv, r, v) in enumerate(systems):
        ens.set_system(s, m, pr, pv, r, v)
    ens.set_starter(starter, mlp_path)
    ens.set_shape(cta, ppt)
    ens.init()
    out = []
    for _ in range(blocks):
        ens.step()
        out.append([(ens.particles(s), ens.counts(s)["n_alive"]) for s in range(len(systems))])
    return out, ens.stats()


def compare(got_blocks, want, T, chaotic=None):
    """Block by block: alive counts, ids, flags, deathtime indices and
    deathtimes exact; positions and velocities of the survivors within
    POS_TOL per 1e3 steps.  `chaotic` names systems of Neptune crossers,
    whose passages just outside three Hill radii magnify rounding
    differences by orders of magnitude within a few hundred steps (the
    oracle's own run from positions one ulp away differs from it by up to
    ~1e-11 after 900 steps, and the kick's float-float pulls carry ~1e-13 of
    each pull per step): there 99 % of the survivors stay within the bound
    and every survivor within 1e-8."""
    chaotic = chaotic or ()
    worst = 0.0
    for b, per_sys in enumerate(got_blocks):
        for s, (got, n_alive) in enumerate(per_sys):
            w, w_alive = want[s][b]
            assert n_alive == w_alive, (b, s)
            assert np.array_equal(got["id"], w["id"]), (b, s)
            assert np.array_equal(got["flags"], w["flags"]), (b, s, np.flatnonzero(got["flags"] != w["flags"])[:8])
            flagged = w["flags"] != 0
            # the oracle keeps the deathtime index of the block a particle left
            # the alive range in, as the ensemble's death record does
            assert np.array_equal(got["deathtime_index"][flagged], w["dti"][flagged]), (b, s)
            assert np.array_equal(got["deathtime"][flagged], w["deathtime"][flagged]), (b, s)
            live = ~flagged
            if live.any():
                tol = POS_TOL * max(1.0, (b + 1) * T / 1000.0)
                er = np.linalg.norm(got["r"] - w["r"], axis=1)[live] / np.linalg.norm(w["r"], axis=1)[live]
                ev = np.linalg.norm(got["v"] - w["v"], axis=1)[live] / np.linalg.norm(w["v"], axis=1)[live]
                if s in chaotic:
                    assert np.quantile(er, 0.99) < tol and np.quantile(ev, 0.99) < tol, \
                        (b, s, np.quantile(er, 0.99), np.quantile(ev, 0.99))
                    assert er.max() < 1e-8 and ev.max() < 1e-8, (b, s, er.max(), ev.max())
                else:
                    assert er.max() < tol and ev.max() < tol, (b, s, er.max(), ev.max())
                    worst = max(worst, er.max())
    return worst


@pytest.fixture(scope="module")
def shaped():
    systems = benchmark_shaped_systems()
    T, blocks = 128, 8                       # 1024 steps
    want = oracle_runs(systems, 180.0, T, blocks, 60.0)
    return systems, T, blocks, want, (2,)       # system 2: the Neptune crossers


@pytest.fixture(scope="module")
def inner_network(tmp_path_factory):
    """A network trained on the inner system's own logged plain solves (the
    drifts with tau^2 >= the log floor), at dt = 20 d."""
    m, pr, pv, r, v = inner_system(4000, seed=77)
    sim = G.Simulation(CFG % (INNER_DT, 16, 60.0))
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v)
    sim.init()
    tr = L.Trainer(4000 * 40 + 1, seed=3)
    tr.set_log_floor(L.LOG_TAU2_FLOOR)
    for _ in range(40):
        tr.log_simulation(sim)
        sim.loop()
    tr.fit_norm()
    tr.train(3000, batch=8192, lr=3e-3, lr_min=1e-5, seed=5)
    path = str(tmp_path_factory.mktemp("mlp") / "inner.bin")
    tr.save(path)
    return tr, path


@pytest.mark.parametrize("starter", ["series", "classic", "learned"])
def test_benchmark_shaped_ensemble_matches_oracle(shaped, inner_network, starter):
    systems, T, blocks, want, chaotic = shaped
    st = {"series": G.STARTER_SERIES, "classic": G.STARTER_CLASSIC, "learned": G.STARTER_LEARNED}[starter]
    got, stats = run_ensemble(systems, 180.0, T, blocks, 60.0, st, inner_network[1] if starter == "learned" else None)
    worst = compare(got, want, T, chaotic)
    print("%s: max rel pos err vs oracle %.2e, borderline tests %d" % (starter, worst, stats["borderline"]))
    assert sum(n for _, n in got[-1]) < sum(len(x[3]) for x in systems)      # particles were removed
    assert stats["borderline"] == 0


def test_learned_network_in_ensemble_matches_oracle(inner_network):
    """The network runs in the inner system's drifts with tau^2 >= 0.01; the
    ensemble with it matches the oracle, and so does the series run on the
    same systems (there the FP32 pre-solve starts those drifts)."""
    tr, path = inner_network
    systems = [inner_system(3000, seed=91)] + benchmark_shaped_systems(seed=55)[:2]
    T, blocks, dt = 128, 8, INNER_DT
    want = oracle_runs(systems, dt, T, blocks, 60.0)
    for st in (G.STARTER_LEARNED, G.STARTER_SERIES):
        got, stats = run_ensemble(systems, dt, T, blocks, 60.0, st, path if st == G.STARTER_LEARNED else None)
        compare(got, want, T)
        assert stats["borderline"] == 0
    # the network's guesses are used: fewer Stumpff evaluations than the
    # classic starter's
    r, v = systems[0][3], systems[0][4]
    ev = {k: L.drift_states(r, v, dt, systems[0][0][0], st, tr)[2].mean()
          for k, st in (("learned", G.STARTER_LEARNED), ("series", G.STARTER_SERIES),
                        ("classic", G.STARTER_CLASSIC))}
    print("inner system, Stumpff evaluations per drift:", ev)
    assert ev["learned"] < ev["classic"]


def test_learned_dispatch_follows_wide_drifts(shaped, inner_network):
    """The learned starter's per-block dispatch.  On the benchmark-shaped
    systems without the crossers no drift reaches tau^2 >= 0.01: only the
    first block launches the network kernel, which on those drifts does the
    series kernel's arithmetic, so the run is bit-identical to the series
    starter's.  In the inner system every block has such drifts and every
    block runs the network."""
    systems, T = [x for k, x in enumerate(shaped[0]) if k != 2], shaped[1]
    blocks = 4
    got, st = run_ensemble(systems, 180.0, T, blocks, 60.0, G.STARTER_LEARNED, inner_network[1])
    ser, ss = run_ensemble(systems, 180.0, T, blocks, 60.0, G.STARTER_SERIES)
    assert st["wide_drifts"] == 0 and st["learned_drifts"] == 0 and ss["wide_drifts"] == 0
    assert st["network_blocks"] == 1 and ss["network_blocks"] == 0
    for b in range(blocks):
        for s, ((g, gn), (w, wn)) in enumerate(zip(got[b], ser[b])):
            assert gn == wn, (b, s)
            for k in ("id", "flags", "deathtime_index"):
                assert np.array_equal(g[k], w[k]), (b, s, k)
            for k in ("r", "v"):
                d = np.abs(g[k] - w[k]).max()
                assert d == 0, (b, s, k, d)
    inner = [inner_system(2000, seed=93)]
    _, si = run_ensemble(inner, INNER_DT, 128, blocks, 60.0, G.STARTER_LEARNED, inner_network[1])
    print("inner system:", si)
    assert si["network_blocks"] == blocks
    assert 0 < si["learned_drifts"] <= si["wide_drifts"]


def test_history_workload_with_learned_starter_matches_oracle(tmp_path, inner_network):
    """The planetary-history + encounter-flagging workload (Sun + Neptune-mass
    planet in yr units, history from the library's planet-only WH at dt =
    0.2 yr with one snapshot per 100 steps, 2,000 Neptune-crossing particles
    a 20-40 au, e < 0.3, Encounter-RH-Factor 3, Time-Block-Size 100) with the
    learned starter, the history evaluated on the device, against the
    oracle's interpolator and block loop."""
    _, path = inner_network
    hist = str(tmp_path / "plhist.out")
    m, pr, pv, r, v = synth.cartesian_state("history-encounters", 2000, seed=8)
    pre = G.Simulation("Time-Step 0.2\nTime-Block-Size 100\nFinal-Time 1e9\nLimit-Particle-Count 0\n"
                       "Input-File x\nOutput-Folder x\n")
    pre.set_planets(m, pr, pv)
    pre.set_particles(np.zeros((0, 3)), np.zeros((0, 3)))
    pre.init()
    pre.write_plhist(hist, begin=True)
    for _ in range(16):
        pre.loop()
        pre.write_plhist(hist)
    del pre
    cfg = ("Time-Step 0.2\nTime-Block-Size 100\nFinal-Time 1e9\nRead-Planet-History 1\nPlanet-History-File %s\n"
           "Encounter-RH-Factor 3\nCull-Radius 0.5\nOuter-Limit 300\nInput-File x\nOutput-Folder x\n" % hist)
    sim = G.Simulation(cfg)
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v)
    sim.set_starter(G.STARTER_LEARNED, path)
    sim.init()
    ex = O.Exec(m, pr, pv, np.arange(len(m)), r, v, np.arange(len(r)), dt=0.2, tbsize=100, outer_r=300.0,
                cull_r=0.5, esf=3.0, interp_path=hist, drift="uv")
    flagged_total = 0
    for b in range(12):
        sim.loop()
        ex.loop()
        assert sim.counts()["n_alive"] == ex.counts()["n_alive"], b
        got = sim.particles()
        want = ex.particles()
        go, wo = np.argsort(got["id"]), np.argsort(want["id"])
        assert np.array_equal(got["id"][go], want["id"][wo])
        assert np.array_equal(got["flags"][go], want["flags"][wo]), b
        assert np.array_equal(got["deathtime"][go], want["deathtime"][wo]), b
        live = want["flags"][wo] == 0
        err = np.linalg.norm(got["r"][go] - want["r"][wo], axis=1) / np.linalg.norm(want["r"][wo], axis=1)
        assert err[live].max() < POS_TOL * max(1.0, (b + 1) * 100 / 1000.0), (b, err[live].max())
        flagged_total += len(sim.flagged()["id"])
    assert flagged_total > 0                 # the Hill-radius flags did fire
    assert sim.stats()["borderline"] == 0
