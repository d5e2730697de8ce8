"""Learned Kepler starter on the GPU: training kernels against the CPU
oracle, logged samples against exact solves, what the trained network saves,
and that the starter never changes the accepted solution.

The time-block kernels run the network only where the series starter is
outside its domain (tau^2 = dt^2 mu / r0^3 >= 0.01) and take the series
starter elsewhere.  The network is trained on that range: the close-eccentric
workload (Sun + a Neptune-mass planet at 30 au; a 2.5-6 au, e 0.1-0.6, so
every drift at dt = 180 d has tau^2 >= 0.0108), logged with the floor
tau^2 >= 0.005.  Simulations also run the scattered-disk distribution (a
log-uniform in 30..1000 au, e up to 0.95, i up to 40 deg), where the series
starter does most drifts.  Outer-Limit 1e5 au.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import glisser_gb300 as G  # noqa: E402
from glisser_gb300 import learned as L  # noqa: E402
from glisser_gb300 import synth  # noqa: E402
from oracle import mlp_oracle as M  # noqa: E402

CFG = ("Time-Step 180\nTime-Block-Size %d\nFinal-Time 1e30\nCull-Radius 0.5\nOuter-Limit 1e5\n"
       "Input-File x\nOutput-Folder x\n")
DT = 180.0


@pytest.fixture(scope="module", autouse=True)
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    G.build()
    G.lib()


def simulation(n, seed, T=64, starter=G.STARTER_SERIES, mlp_path=None, workload="scattered-disk"):
    m, pr, pv, r, v = synth.cartesian_state(workload, n, seed)
    sim = G.Simulation(CFG % T)
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v)
    sim.set_starter(starter, mlp_path)
    sim.init()
    return sim, (m, r, v)


@pytest.fixture(scope="module")
def trained(tmp_path_factory):
    tr = L.Trainer(1 << 18, seed=5)
    tr.set_log_floor(L.LOG_TAU2_FLOOR)
    sim, state = simulation(8192, seed=11, workload="close-eccentric")
    losses = L.train_on_simulation(sim, tr, blocks=16, steps=3000, batch=8192, lr=3e-3, lr_min=1e-5, seed=3)
    path = str(tmp_path_factory.mktemp("mlp") / "starter.bin")
    tr.save(path)
    return tr, losses, state, path


def features(r, v, mu, dt):
    r0 = np.linalg.norm(r, axis=1)
    u = (r * v).sum(1)
    alpha = 2 * mu / r0 - (v * v).sum(1)
    tau = dt * np.sqrt(mu / r0 ** 3)
    return np.stack([np.log(tau), u / np.sqrt(mu * r0), alpha * r0 / mu], 1), r0, u, alpha


def exact_s(dt, r0, u, mu, alpha, s):
    """Newton on the universal Kepler equation with closed-form Stumpff
    functions (float64), from a nearby start."""
    for _ in range(30):
        x = alpha * s * s
        sx = np.sqrt(np.abs(x))
        with np.errstate(invalid="ignore", divide="ignore"):
            c2 = np.where(x > 0, (1 - np.cos(sx)) / x, (np.cosh(sx) - 1) / -x)
            c3 = np.where(x > 0, (sx - np.sin(sx)) / sx ** 3, (np.sinh(sx) - sx) / sx ** 3)
        small = np.abs(x) < 1e-3
        c2 = np.where(small, 0.5 - x / 24 + x * x / 720, c2)
        c3 = np.where(small, 1 / 6 - x / 120 + x * x / 5040, c3)
        g1 = s * (1 - x * c3)
        g2 = s * s * c2
        g3 = s ** 3 * c3
        f = r0 * g1 + u * g2 + mu * g3 - dt
        fp = r0 * (1 - x * c2) + u * g1 + mu * g2
        s = s - f / fp
    return s


def test_gradients_match_oracle():
    rng = np.random.default_rng(4)
    tr = L.Trainer(1024, seed=9)
    norm = dict(in_mean=[-6.5, 0.0, 1.1], in_scale=[0.45, 2.2, 1.7], x_lo=[-30, -5, -1], x_hi=[5, 5, 5],
                out_mean=0.002, out_scale=0.015)
    tr.norm = norm
    p = M.init_params(9)
    p[M.OFF_B1:M.OFF_W2] = rng.normal(0, 0.2, 32)
    p[M.OFF_B2:M.OFF_W3] = rng.normal(0, 0.2, 32)
    tr.params = p
    n = 1000                      # not a multiple of the 128-sample tile
    feat = np.stack([rng.uniform(-10, 0, n), rng.uniform(-1, 1, n), rng.uniform(0, 2, n)], 1).astype(np.float32)
    target = rng.normal(0.0, 0.03, n).astype(np.float32)
    g_gpu, loss_gpu = tr.gradients(feat, target)
    nm = tr.norm
    loss, g = M.loss_and_grad(p, nm, feat.astype(np.float64), target.astype(np.float64))
    assert abs(loss_gpu - loss) <= 1e-5 * loss
    for a, b in ((M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
                 (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.NPARAM)):
        d = np.linalg.norm(g_gpu[a:b] - g[a:b]) / np.linalg.norm(g[a:b])
        assert d < 1e-4, (a, d)      # FP32 accumulation and fast exp against float64


def test_logged_samples_are_plain_solves(trained):
    tr, _, (m, r, v), _ = trained
    mu = m[0]
    n = len(r)
    feat, z = tr.get_samples(0, n)           # first log: the initial states, in id order
    f_ref, r0, u, alpha = features(r, v, mu, DT)
    assert np.allclose(feat, f_ref, rtol=2e-6, atol=2e-6)
    tau = np.exp(f_ref[:, 0])
    s0 = DT / r0 * np.exp(z.astype(np.float64) * tau)
    s = exact_s(DT, r0, u, mu, alpha, s0)
    z_ref = np.log(s * r0 / DT) / tau
    assert np.all(np.isfinite(z))
    assert np.max(np.abs(z - z_ref) / (1e-3 + np.abs(z_ref))) < 1e-5
    count, evals = tr.samples()
    assert 15 * n < count <= 16 * n and evals > count


def test_training_converges(trained):
    _, losses, _, _ = trained
    assert np.all(np.isfinite(losses))
    assert losses[-200:].mean() < 1e-2 * losses[:10].mean()


def test_inference_matches_oracle(trained):
    tr, _, _, _ = trained
    feat, _ = tr.get_samples(5 * 8192, 4096)
    y_gpu = tr.predict(feat)
    y_ref = M.predict(tr.params, tr.norm, feat.astype(np.float64))
    ok = np.isfinite(y_ref)
    assert np.array_equal(np.isfinite(y_gpu), ok)
    # the GPU runs the time-block kernels' inference (mlp_forward: FP32 FMAs,
    # the inputs and the hidden activations each read as a BF16 hi + lo
    # pair).  The FP32 values and the oracle's float64 ones can round to
    # different pairs at a rounding boundary (2^-17 of the value), for the
    # inputs and for the activations alike, hence the looser bound on the few
    # largest differences.
    scale = float(tr.norm["out_scale"])
    d = np.abs(y_gpu[ok] - y_ref[ok])
    assert np.quantile(d, 0.999) < 3e-5 * scale + 1e-6
    assert d.max() < 3e-4 * scale + 1e-6


def test_learned_starter_saves_newton_passes(trained):
    """Where the network runs (every drift of held-out close-eccentric
    states) its guess needs fewer Stumpff evaluations than the reference's
    classic starter (about two); most are accepted on the first evaluation
    by predicted acceptance (the reverted correction provably lands within
    the tolerance).  The series rule there is the FP32 Kepler pre-solve.  On
    the scattered disk the series starter does almost every drift for both
    (orders 2-4 in float-float, accepted on the first evaluation)."""
    tr, _, _, _ = trained
    for workload in ("close-eccentric", "scattered-disk"):
        m, pr, pv, r, v = synth.cartesian_state(workload, 8192, seed=12)     # held out
        mu = m[0]
        out = {}
        for name, st in (("classic", G.STARTER_CLASSIC), ("learned", G.STARTER_LEARNED),
                         ("series", G.STARTER_SERIES)):
            out[name] = L.drift_states(r, v, DT, mu, st, tr)
        ev = {k: o[2].mean() for k, o in out.items()}
        print(workload, "mean Stumpff evaluations per drift:", ev)
        assert ev["learned"] < ev["classic"] - 0.5
        if workload == "scattered-disk":
            assert ev["series"] < 1.05 and ev["learned"] < 1.05
        for k in ("learned", "series"):
            assert np.array_equal(out[k][3], out["classic"][3])
            rr = np.linalg.norm(out[k][0] - out["classic"][0], axis=1) / np.linalg.norm(out["classic"][0], axis=1)
            assert rr.max() < 1e-12, (k, rr.max())


@pytest.mark.parametrize("workload,T,blocks", [("scattered-disk", 256, 4), ("close-eccentric", 128, 2)])
def test_simulation_learned_matches_series(trained, workload, T, blocks):
    """The same simulation with the learned and the series starter: flags
    and counts identical, positions within 1e-10 (1024 steps of the scattered
    disk; 256 steps of the close-eccentric workload, whose 8-30 steps per
    orbit magnify rounding differences fastest)."""
    _, _, _, path = trained
    runs = {}
    for st in (G.STARTER_SERIES, G.STARTER_LEARNED):
        sim, _ = simulation(2048, seed=13, T=T, starter=st, mlp_path=path if st == G.STARTER_LEARNED else None,
                            workload=workload)
        for _ in range(blocks):
            sim.loop()
        p = sim.particles()
        o = np.argsort(p["id"])
        runs[st] = ({k: p[k][o] for k in ("r", "v", "flags", "id")}, sim.counts(), sim.stats())
    a, b = runs[G.STARTER_SERIES], runs[G.STARTER_LEARNED]
    assert np.array_equal(a[0]["flags"], b[0]["flags"])
    assert a[1] == b[1]
    live = a[0]["flags"] == 0
    err = np.linalg.norm(a[0]["r"] - b[0]["r"], axis=1) / np.linalg.norm(a[0]["r"], axis=1)
    assert err[live].max() < 1e-10, err[live].max()
    assert a[2]["particle_steps"] == b[2]["particle_steps"]
    # both workloads have drifts with tau^2 >= 0.01 in every block, where the
    # learned run's network kernel runs (the network, trained on the
    # close-eccentric workload, starts those of them inside its box)
    assert b[2]["network_blocks"] == blocks and a[2]["network_blocks"] == 0
    assert 0 < b[2]["wide_drifts"] and b[2]["learned_drifts"] <= b[2]["wide_drifts"]
    if workload == "close-eccentric":
        assert b[2]["learned_drifts"] > 0


def test_ensemble_learned_matches_series_and_is_launch_invariant(trained):
    _, _, _, path = trained
    systems = []
    for s in range(3):
        wl = "close-eccentric" if s == 1 else "scattered-disk"
        m, pr, pv, r, v = synth.cartesian_state(wl, [300, 900, 129][s], seed=20 + s)
        systems.append((m, pr, pv, r, v))

    def run(starter, cta=128, ppt=1, graph=True):
        ens = G.Ensemble(CFG % 128, len(systems))
        for s, (m, pr, pv, r, v) in enumerate(systems):
            ens.set_system(s, m, pr, pv, r, v)
        ens.set_starter(starter, path if starter == G.STARTER_LEARNED else None)
        ens.set_shape(cta, ppt)
        ens.set_graph(graph)
        ens.init()
        for _ in range(4):
            ens.step()
        return [ens.particles(s) for s in range(len(systems))]

    ser = run(G.STARTER_SERIES)
    lrn = run(G.STARTER_LEARNED)
    lrn2 = run(G.STARTER_LEARNED, 64, 2, False)
    for s in range(len(systems)):
        assert np.array_equal(ser[s]["flags"], lrn[s]["flags"])
        err = np.linalg.norm(ser[s]["r"] - lrn[s]["r"], axis=1) / np.linalg.norm(ser[s]["r"], axis=1)
        assert err.max() < 1e-10
        assert np.array_equal(lrn[s]["flags"], lrn2[s]["flags"])
        if s != 1:
            # the scattered-disk systems take the same arithmetic whatever the
            # launch shape; on the close-eccentric system the warp-uniform
            # Stumpff tiers depend on which particles share a warp, so
            # another shape rounds differently there
            assert np.array_equal(lrn[s]["r"], lrn2[s]["r"])
        else:
            err = np.linalg.norm(lrn2[s]["r"] - lrn[s]["r"], axis=1) / np.linalg.norm(lrn[s]["r"], axis=1)
            assert err.max() < 1e-10


def test_bad_weights_file_is_rejected(tmp_path):
    p = tmp_path / "bad.bin"
    p.write_bytes(b"GLMLP000" + bytes(100))
    sim = G.Simulation(CFG % 64)
    with pytest.raises(G.GlisserError):
        sim.set_starter(G.STARTER_LEARNED, str(p))
    assert os.path.exists(p)


def test_outside_the_training_box_the_series_rule_runs(trained, tmp_path):
    """Drifts whose features fall outside the network's training box take
    the series rule (the series starter, or the FP32 pre-solve where tau^2 >=
    0.01): the same arithmetic as the series starter, bit for bit, in the
    drift routine and in the time-block kernel."""
    tr, _, _, _ = trained
    nm = tr.norm
    narrow = L.Trainer(16, seed=1)
    narrow.params = tr.params
    narrow.norm = dict(nm, x_lo=np.array([50.0, 50.0, 50.0]), x_hi=np.array([51.0, 51.0, 51.0]))
    for wl in ("scattered-disk", "close-eccentric"):
        m, pr, pv, r, v = synth.cartesian_state(wl, 2048, seed=14)
        a = L.drift_states(r, v, DT, m[0], G.STARTER_LEARNED, narrow)
        b = L.drift_states(r, v, DT, m[0], G.STARTER_SERIES)
        assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3])
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    path = str(tmp_path / "narrow.bin")
    narrow.save(path)
    finals = []
    for st in (G.STARTER_LEARNED, G.STARTER_SERIES):
        sim, _ = simulation(1024, seed=15, T=128, starter=st, mlp_path=path if st == G.STARTER_LEARNED else None,
                            workload="close-eccentric")
        for _ in range(2):
            sim.loop()
        finals.append(sim.particles())
    assert np.array_equal(finals[0]["r"], finals[1]["r"]) and np.array_equal(finals[0]["flags"], finals[1]["flags"])


def test_tighter_kepler_tolerance(trained):
    """The scattered-disk workload's Newton tolerance, |f| < 1e-14 dt: the
    same flags, positions within 1e-10 of the default-tolerance run, at most
    a few more Stumpff evaluations per step; out-of-range tolerances are
    refused."""
    _, _, _, path = trained
    runs = {}
    for tol in (None, 1e-14):
        sim, _ = simulation(2048, seed=16, T=128)
        if tol:
            sim.set_kepler_tolerance(tol)
        for _ in range(4):
            sim.loop()
        p = sim.particles()
        o = np.argsort(p["id"])
        runs[tol] = (p["r"][o], p["flags"][o], sim.stats())
    a, b = runs[None], runs[1e-14]
    assert np.array_equal(a[1], b[1])
    live = a[1] == 0
    err = np.linalg.norm(a[0] - b[0], axis=1) / np.linalg.norm(a[0], axis=1)
    assert err[live].max() < 1e-10
    ev_a = a[2]["kepler_evals"] / a[2]["particle_steps"]
    ev_b = b[2]["kepler_evals"] / b[2]["particle_steps"]
    assert ev_a <= ev_b < ev_a + 0.2
    sim, _ = simulation(16, seed=17, T=16)
    with pytest.raises(G.GlisserError):
        sim.set_kepler_tolerance(1e-20)


LD = np.longdouble


def stumpff_ld(x):
    """c0..c3 of x in long double: the series on x / 4^n (|x / 4^n| < 0.1)
    and the double-angle rebuild."""
    y = x.copy()
    n = np.zeros(x.shape, np.int64)
    for _ in range(200):
        big = np.abs(y) >= 0.1
        if not big.any():
            break
        y[big] /= 4
        n[big] += 1
    c2 = np.zeros_like(y)
    c3 = np.zeros_like(y)
    t2 = np.full_like(y, LD(1) / 2)
    t3 = np.full_like(y, LD(1) / 6)
    for k in range(16):
        c2 += t2
        c3 += t3
        t2 = t2 * -y / ((2 * k + 3) * (2 * k + 4))
        t3 = t3 * -y / ((2 * k + 4) * (2 * k + 5))
    c1 = 1 - y * c3
    c0 = 1 - y * c2
    for i in range(int(n.max(initial=0))):
        m = n > i
        c3, c2, c1, c0 = (np.where(m, (c2 + c0 * c3) / 4, c3), np.where(m, c1 * c1 / 2, c2),
                          np.where(m, c0 * c1, c1), np.where(m, 2 * c0 * c0 - 1, c0))
    return c0, c1, c2, c3


def drift_ld(r, v, dt, mu):
    """One Kepler drift in long double: universal-variable Kepler equation
    solved by bisection (f is increasing, f' = |r| > 0) and Newton polish,
    then the f and g functions."""
    r = r.astype(LD)
    v = v.astype(LD)
    dt = LD(dt)
    mu = LD(mu)
    r0 = np.sqrt((r * r).sum(1))
    u = (r * v).sum(1)
    alpha = 2 * mu / r0 - (v * v).sum(1)

    def kep(s):
        c0, c1, c2, c3 = stumpff_ld(alpha * s * s)
        g = (c0, s * c1, s * s * c2, s * s * s * c3)
        return r0 * g[1] + u * g[2] + mu * g[3] - dt, r0 * g[0] + u * g[1] + mu * g[2], g

    lo = np.zeros_like(r0)
    hi = dt / r0
    for _ in range(200):
        f, _, _ = kep(hi)
        low = f <= 0
        if not low.any():
            break
        lo = np.where(low, hi, lo)
        hi = np.where(low, 2 * hi, hi)
    for _ in range(80):
        mid = (lo + hi) / 2
        f, _, _ = kep(mid)
        lo = np.where(f <= 0, mid, lo)
        hi = np.where(f <= 0, hi, mid)
    s = (lo + hi) / 2
    for _ in range(2):
        f, fp, _ = kep(s)
        s = s - f / fp
    _, _, (_, g1, g2, g3) = kep(s)
    fr = 1 - mu * g2 / r0
    gr = dt - mu * g3
    rn = fr[:, None] * r + gr[:, None] * v
    rr = np.sqrt((rn * rn).sum(1))
    fd = -mu * g1 / (rr * r0)
    gd = 1 - mu * g2 / rr
    vn = fd[:, None] * r + gd[:, None] * v
    return rn, vn


def test_one_drift_matches_long_double_solution(trained):
    """One drift of 4096 scattered-disk states with each starter, at the
    workload's step and at 10x and 100x it (steps through pericentre of the
    eccentric orbits), and of 4096 close-eccentric states at the workload's
    step (every drift started by the network or the FP32 pre-solve), against
    the long-double solution: every acceptance path (the residual test, the
    predicted acceptance with its third-order fold, the Laguerre fallback)
    lands at FP64 rounding, and the starters agree to rounding.  With tau ~ 1
    (100x on the scattered disk, the close-eccentric drifts) the Stumpff
    functions' argument quartering costs a few more bits, in the same way for
    every starter, and the result is still well inside the FP64 restatement
    of the reference's drift (no fold of the last correction)."""
    tr, _, _, _ = trained
    bounds = {("scattered-disk", DT): 1e-15, ("scattered-disk", 10 * DT): 2e-15,
              ("scattered-disk", 100 * DT): 2e-13, ("close-eccentric", DT): 2e-13}
    from oracle import oracle as O
    O.build()
    cases = [("scattered-disk", dt) for dt in (DT, 10 * DT, 100 * DT)] + [("close-eccentric", DT)]
    for wl, dt in cases:
        m, pr, pv, r, v = synth.cartesian_state(wl, 4096, seed=21)
        mu = m[0]
        rl, vl = drift_ld(r, v, dt, mu)
        nr = np.sqrt((rl * rl).sum(1))
        nv = np.sqrt((vl * vl).sum(1))
        rl, vl = rl.astype(np.float64), vl.astype(np.float64)
        errs = {}
        for name, st in (("classic", G.STARTER_CLASSIC), ("series", G.STARTER_SERIES),
                         ("learned", G.STARTER_LEARNED)):
            gr, gv, ev, fl = L.drift_states(r, v, dt, mu, st, tr)
            assert not fl.any(), (name, dt)
            er = (np.linalg.norm(gr - rl, axis=1) / nr).astype(np.float64)
            evv = (np.linalg.norm(gv - vl, axis=1) / nv).astype(np.float64)
            errs[name] = (er.max(), np.quantile(er, 0.99), evv.max(), ev.mean())
        orr, ovv = r.copy(), v.copy()
        O.uv_drift(orr, ovv, dt, mu)
        errs["oracle"] = (float((np.linalg.norm(orr - rl, axis=1) / nr).max()), 0.0,
                          float((np.linalg.norm(ovv - vl, axis=1) / nv).max()), 0.0)
        for k, e in errs.items():
            print("%s dt %6g %-8s r max %.2e p99 %.2e  v max %.2e  evals %.3f" % ((wl, dt, k) + e))
        bound = bounds[(wl, dt)]
        for k in ("classic", "series", "learned"):
            assert errs[k][0] < bound and errs[k][2] < bound, (wl, dt, k, errs[k])
            assert errs[k][0] <= 2 * errs["series"][0] + 1e-15, (dt, k, errs[k], errs["series"])
            assert errs[k][0] <= max(errs["oracle"][0], 5e-16) and errs[k][2] <= max(errs["oracle"][2], 5e-16), \
                (dt, k, errs)
        if wl == "scattered-disk" and dt < 100 * DT:
            assert errs["series"][3] < 1.01, errs["series"]
