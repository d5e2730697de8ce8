"""GPU parity of the time-block kernel and the executor against the oracle.

The oracle (oracle/glisser_oracle.c, pinned to the compiled reference by
test_oracle_pin.py) runs the reference's own algorithm: the MVS elliptic drift
of src/wh.cu with its flag rules.  The device kernel drifts with the
universal-variable solver, so positions agree to rounding-level differences
amplified by the dynamics; the bound is the one the spec states, 1e-10
relative after ~1e3 steps.  Flags, deathtime indices, ids and alive counts are
compared exactly.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import glisser_gb300 as G  # noqa: E402

GOLD = os.path.join(os.path.dirname(__file__), "golden")
POS_TOL = 1e-10           # relative position agreement after ~1e3 steps
CASES = ["neptune_t128", "giants_t256", "flags_t64", "hill_t64", "interp_t50", "formats_run"]


@pytest.fixture(scope="module", autouse=True)
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    G.build()
    G.lib()


def load(case):
    d = np.load(os.path.join(GOLD, case + ".npz"))
    cfg = dict(line.split(" ", 1) for line in str(d["config"]).split("\n"))
    return d, cfg


def oracle_exec(d, cfg):
    kw = dict(t0=0.0, dt=float(cfg["Time-Step"]), tbsize=int(cfg["Time-Block-Size"]),
              outer_r=float(cfg.get("Outer-Limit", 300)), cull_r=float(cfg.get("Cull-Radius", 0.5)),
              esf=float(cfg.get("Encounter-RH-Factor", 0)))
    if "Planet-History-File" in cfg:
        kw["interp_path"] = os.path.join(GOLD, "plhist_yr.bin")
    n = len(d["r0"])
    return O.Exec(d["pl_m"], d["pl_r"], d["pl_v"], np.arange(len(d["pl_m"])), d["r0"], d["v0"], np.arange(n),
                  ref_quirks=False, **kw)


def by_id(p):
    o = np.argsort(p["id"])
    return {k: np.asarray(v)[o] for k, v in p.items()}


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("starter,kick", [(G.STARTER_SERIES, G.KICK_FLOAT_FLOAT), (G.STARTER_CLASSIC, G.KICK_FLOAT_FLOAT),
                                          (G.STARTER_SERIES, G.KICK_FP64)])
def test_kernel_block_parity(case, starter, kick):
    """The C-ABI time-block kernel, block after block, against the oracle,
    with the float-float kick and with the FP64 kick.  No radius test of
    these fixtures is threshold-borderline (glisser_handoff.borderline), so
    the flags cannot depend on the kick's arithmetic."""
    from gpu_util import DevParticles, DevPlanetBlock, DevHandoff, timeblock, rel_err
    d, cfg = load(case)
    ex = oracle_exec(d, cfg)
    p0 = ex.particles()
    parts = DevParticles(p0["r"], p0["v"], p0["a"], p0["flags"], p0["id"])
    outer = float(cfg.get("Outer-Limit", 300))
    ho = DevHandoff(parts.n)
    steps = 0
    for b in range(int(d["nblocks"])):
        blk = ex.planet_block()
        c = ex.counts()
        dev_blk = DevPlanetBlock(blk["h0_log"], blk["r_log"], blk["m"], blk["id"], blk["rh"])
        before = by_id(parts.host())["flags"].copy()
        res = timeblock(parts, dev_blk, c["dt"], outer, starter=starter, handoff=ho, kick=kick)
        assert res["status"] == 0
        assert res["borderline"] == 0, b
        ex.loop()
        steps += blk["log_len"]
        got = by_id(parts.host())
        want = by_id(ex.particles())
        assert np.array_equal(got["id"], want["id"])
        assert np.array_equal(got["flags"], want["flags"]), (b, np.nonzero(got["flags"] != want["flags"]))
        changed = got["flags"] != before
        assert np.array_equal(got["dti"][changed], want["dti"][changed])
        assert sorted(res["id"].tolist()) == sorted(got["id"][changed].tolist())
        err = rel_err(got["r"], want["r"])
        assert err.max() < POS_TOL * max(1.0, steps / 1000.0), (b, err.max())
        verr = rel_err(got["v"], want["v"])
        assert verr.max() < POS_TOL * max(1.0, steps / 1000.0), (b, verr.max())


@pytest.mark.parametrize("kick", [G.KICK_FLOAT_FLOAT, G.KICK_FP64])
def test_plain_giants_against_oracle_both_kicks(kick):
    """The plain-giants workload (Sun + four giants, particles near the
    Neptune 3:1, a 53-57 au, e < 0.3, i < 10 deg; dt = 180 d) on a 4,096-
    particle sample over 1,024 steps through the executor, with each kick:
    flags and survivors equal to the oracle's, positions within 1e-10
    relative, no threshold-borderline radius test; the two kicks agree with
    each other to the same bound."""
    from glisser_gb300 import synth
    m, pr, pv, r, v = synth.cartesian_state("plain-giants", 4096, seed=1000)
    cfg = ("Time-Step 180\nTime-Block-Size 1024\nFinal-Time 1e30\nCull-Radius 0.5\nOuter-Limit 300\n"
           "Input-File unused\nOutput-Folder unused\n")
    sim = G.Simulation(cfg)
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v)
    sim.set_kick(kick)
    sim.init()
    sim.loop()
    ex = O.Exec(m, pr, pv, np.arange(len(m)), r, v, np.arange(len(r)), dt=180.0, tbsize=1024)
    ex.loop()
    got, want = by_id(sim.particles()), by_id(ex.particles())
    assert np.array_equal(got["flags"], want["flags"])
    assert sim.counts()["n_alive"] == ex.counts()["n_alive"]
    live = want["flags"] == 0
    err = np.linalg.norm(got["r"] - want["r"], axis=1) / np.linalg.norm(want["r"], axis=1)
    print("kick %d: max rel pos err vs oracle %.2e" % (kick, err[live].max()))
    assert err[live].max() < POS_TOL * 1.024
    assert sim.stats()["borderline"] == 0


def test_partition_stable_three_way():
    from gpu_util import DevParticles
    rng = np.random.default_rng(1)
    n = 100_003
    flags = np.zeros(n, np.uint16)
    pick = rng.random(n)
    flags[pick < 0.2] = 0x0101
    flags[(pick >= 0.2) & (pick < 0.3)] = 0x0080
    flags[(pick >= 0.3) & (pick < 0.35)] = 0x0002
    ids = rng.permutation(n).astype(np.uint32)
    r = rng.normal(size=(n, 3)); v = rng.normal(size=(n, 3)); a = rng.normal(size=(n, 3))
    src = DevParticles(r, v, a, flags, ids)
    dst = DevParticles(np.zeros_like(r), np.zeros_like(v), np.zeros_like(a), np.zeros(n, np.uint16), np.zeros(n))
    scratch = torch.zeros(G.partition_scratch_bytes(n), dtype=torch.uint8, device="cuda")
    counts = torch.zeros(2, dtype=torch.int32, device="cuda")
    G.partition(src.view, dst.view, n, scratch.data_ptr(), counts.data_ptr(), counts.data_ptr() + 4)
    out = dst.host()
    cat = np.where(flags == 0, 0, np.where((flags & 0xFE) == 0, 1, 2))
    order = np.argsort(cat, kind="stable")
    assert np.array_equal(out["id"], ids[order])
    assert np.array_equal(out["flags"], flags[order])
    assert np.array_equal(out["r"], r[order])
    c = counts.cpu().numpy()
    assert c[0] == (cat == 0).sum() and c[1] == (cat == 1).sum()
