"""Resolve-Encounters on the GPU: the time-block kernel's rollback mode and
the executor's SWIFT hand-off against the reference.

The reference side is tests/golden/encounters_t50.npz: the reference's own
SwiftEncounterIntegrator (src/swift.cpp) driven by the restated executor loop
(src/executor.cu:470-596, 598-764, 766-877) in oracle/ref_driver.cu, with
SWIFT stood in for by tests/fake_swift.py.  The same stand-in runs here, so
every difference is the library's: counts after every block and the lines of
encounter.out exactly; final flags, deathtimes and SWIFT's status arrays
exactly; positions and velocities to 1e-9 relative (the block integrator's
universal-variable drift against the reference's elliptic one, ~1.2e3
steps); the files of every SWIFT call byte for byte where they do not carry
particle states, to 1e-9 where they do.
"""
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import glisser_gb300 as G  # noqa: E402
from oracle import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
sys.path.insert(0, HERE)
import fake_swift  # noqa: E402

TOL = 1e-9


@pytest.fixture(scope="module", autouse=True)
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    G.build()
    G.lib()


def by_id(p):
    o = np.argsort(p["id"])
    return {k: np.asarray(v)[o] for k, v in p.items()}


def rel(x, y):
    return np.abs(x - y).max() / max(np.abs(y).max(), 1e-300)


# ---------------------------------------------------------------------------
# kernel: GLISSER_ENCOUNTERS_ROLLBACK


def test_rollback_mode_keeps_block_start_state():
    """Rollback leaves a particle flagged into an encounter at its
    block-start r, v; everything else is the keep-mode result bit for bit."""
    from gpu_util import DevParticles, DevPlanetBlock, timeblock
    d = np.load(os.path.join(GOLD, "hill_t64.npz"))
    cfg = dict(line.split(" ", 1) for line in str(d["config"]).split("\n"))
    n = len(d["r0"])
    ex = O.Exec(d["pl_m"], d["pl_r"], d["pl_v"], np.arange(len(d["pl_m"])), d["r0"], d["v0"], np.arange(n),
                ref_quirks=False, t0=0.0, dt=float(cfg["Time-Step"]), tbsize=int(cfg["Time-Block-Size"]),
                outer_r=300.0, cull_r=float(cfg["Cull-Radius"]), esf=float(cfg["Encounter-RH-Factor"]))
    seen = 0
    for _ in range(int(d["nblocks"])):
        p0 = ex.particles()
        blk = ex.planet_block()
        dev_blk = DevPlanetBlock(blk["h0_log"], blk["r_log"], blk["m"], blk["id"], blk["rh"])
        keep = DevParticles(p0["r"], p0["v"], p0["a"], p0["flags"], p0["id"])
        roll = DevParticles(p0["r"], p0["v"], p0["a"], p0["flags"], p0["id"])
        rk = timeblock(keep, dev_blk, ex.counts()["dt"], 300.0, encounters=G.ENCOUNTERS_KEEP)
        rr = timeblock(roll, dev_blk, ex.counts()["dt"], 300.0, encounters=G.ENCOUNTERS_ROLLBACK)
        a, b = keep.host(), roll.host()
        assert rk["status"] == 0 and rr["status"] == 0
        assert np.array_equal(a["flags"], b["flags"]) and np.array_equal(a["dti"], b["dti"])
        assert sorted(rk["id"].tolist()) == sorted(rr["id"].tolist())
        enc = (b["flags"] != 0) & ((b["flags"] & 0xFE) == 0)
        seen += int(np.count_nonzero(enc & (p0["flags"] == 0)))
        for k in ("r", "v"):
            np.testing.assert_array_equal(b[k][enc], p0[k][enc])
            np.testing.assert_array_equal(b[k][~enc], a[k][~enc])
        np.testing.assert_array_equal(b["a"], a["a"])
        ex.loop()
    assert seen > 0


def test_rollback_mode_validated():
    from gpu_util import DevParticles, DevPlanetBlock
    parts = DevParticles(np.ones((4, 3)) * 30, np.zeros((4, 3)), np.zeros((4, 3)), np.zeros(4), np.arange(4))
    blk = DevPlanetBlock(np.zeros((2, 3)), np.zeros((2, 0, 3)), [1.0], [0], [0.1])
    from gpu_util import DevHandoff
    ho = DevHandoff(4)
    sp = G.StepParams(1.0, 300.0, G.STARTER_SERIES, 3, 0)
    with pytest.raises(G.GlisserError):
        G.integrate_timeblock(parts.view, parts.n, blk.view, sp, ho.view)


# ---------------------------------------------------------------------------
# executor: the SWIFT hand-off


def make_sim(d, tmp_path, swift):
    out = tmp_path / "out"
    out.mkdir(exist_ok=True)
    plh = os.path.join(GOLD, "plhist_yr.bin")
    cfg = (str(d["config"]) + "\nPlanet-History-File %s\nSwift-Path %s\nOutput-Folder %s\nInput-File unused\n"
           % (plh, swift, out))
    sim = G.Simulation(cfg)
    sim.set_planets(d["pl_m"], d["pl_r"], d["pl_v"], np.arange(len(d["pl_m"])))
    sim.set_particles(d["r0"], d["v0"], d["id0"])
    return sim, out


def parse_log(text):
    out = []
    for line in text.strip().split("\n"):
        if line.strip():
            i, kind, t = line.split()
            out.append((int(i), kind, float(t)))
    return sorted(out)


def parse_stat(text):
    lines = [l for l in text.strip("\n").split("\n")]
    if not text.strip():
        return {}
    return {int(lines[q]): ([int(x) for x in lines[q + 1].split()], np.array([float(x) for x in lines[q + 2].split()]))
            for q in range(0, len(lines), 3)}


def parse_tp(b):
    tok = b.decode().split()
    n = int(tok[0])
    per = (len(tok) - 1) // n if n else 0
    return n, np.array([[float(x) for x in tok[1 + k * per:7 + k * per]] for k in range(n)])


def parse_tpout(b):
    lines = b.decode().strip().split("\n")
    n = int(lines[0])
    st = np.array([[float(x) for x in lines[1 + 3 * k].split()] for k in range(n)])
    ist = [lines[2 + 3 * k] for k in range(n)]
    return st, ist


def test_resolve_encounters_matches_reference(tmp_path, monkeypatch):
    d = np.load(os.path.join(GOLD, "encounters_t50.npz"))
    swift = fake_swift.wrapper(str(tmp_path))
    arch = tmp_path / "archive"
    monkeypatch.setenv("FAKE_SWIFT_ARCHIVE", str(arch))
    sim, out = make_sim(d, tmp_path, swift)
    sim.init()
    lines = []
    for b in range(int(d["nblocks"])):
        safe, _, _ = sim.loop()
        t, _, host_alive, n_enc = d["counts"][b]
        c = sim.counts()
        assert sim.t == t, (b, sim.t, t)
        assert (c["n_alive"], c["n_encounter"]) == (host_alive, n_enc), b
        if safe:
            assert c["n_encounter"] == 0
        f = sim.flagged()
        lines += [(int(i), "death" if fl & 0x80 else "encounter", sim.t) for i, fl in zip(f["id"], f["flags"])]
    assert sorted(lines) == parse_log(str(d["encounter_log"]))

    got = by_id(sim.particles())
    assert np.array_equal(got["id"], np.sort(d["out_id"]))
    o = np.argsort(d["out_id"])
    assert np.array_equal(got["flags"], d["out_flags"][o])
    assert np.array_equal(got["deathtime"], d["out_deathtime"][o])
    assert rel(got["r"], d["out_r"][o]) < TOL
    assert rel(got["v"], d["out_v"][o]) < TOL

    sim.finish()
    ours = parse_stat(open(out / "stat.out").read())
    ref = parse_stat(str(d["stat_out"]))
    assert sorted(ours) == sorted(ref)
    for pid in ref:
        assert ours[pid][0] == ref[pid][0], pid
        np.testing.assert_allclose(ours[pid][1], ref[pid][1], rtol=TOL, atol=0)

    names = sorted(os.listdir(arch))
    assert names == sorted(str(x) for x in d["archive_names"])
    for nm in names:
        def mine(tag):
            return open(arch / nm / tag, "rb").read()

        def theirs(tag):
            return d["arch_%s_%s" % (nm, tag)].tobytes()
        assert mine("param") == theirs("param"), nm
        assert mine("hist") == theirs("hist"), nm
        n1, s1 = parse_tp(mine("tp"))
        n2, s2 = parse_tp(theirs("tp"))
        assert n1 == n2 and rel(s1, s2) < TOL, nm
        o1, i1 = parse_tpout(mine("tpout"))
        o2, i2 = parse_tpout(theirs("tpout"))
        assert i1 == i2 and rel(o1, o2) < TOL, nm
    assert (out / "swift_data" / "stdout0").exists()


def test_initial_encounter_particle_goes_to_swift(tmp_path, monkeypatch):
    """A particle that starts flagged in an encounter is not advanced by the
    first block, is reported as an encounter after it and is handed to SWIFT
    from its initial state."""
    d = np.load(os.path.join(GOLD, "encounters_t50.npz"))
    swift = fake_swift.wrapper(str(tmp_path))
    arch = tmp_path / "archive"
    monkeypatch.setenv("FAKE_SWIFT_ARCHIVE", str(arch))
    sim, _ = make_sim(d, tmp_path, swift)
    flags = np.zeros(len(d["r0"]), np.uint16)
    flags[5] = 0x0201
    sim.set_particles(d["r0"], d["v0"], d["id0"], flags=flags)
    sim.init()
    sim.loop()
    f = sim.flagged()
    pid = int(d["id0"][5])
    assert pid in f["id"].tolist()
    assert int(f["flags"][f["id"].tolist().index(pid)]) == 0x0201
    p = by_id(sim.particles())
    k = int(np.searchsorted(p["id"], pid))
    np.testing.assert_array_equal(p["r"][k], d["r0"][5])
    sim.loop()
    tp = [n for n in os.listdir(arch) if n.endswith("_tp0")]
    assert tp, "no SWIFT call"
    _, st = parse_tp(open(arch / sorted(tp)[0] / "tp", "rb").read())
    assert any(np.array_equal(row[:3], d["r0"][5]) for row in st)


def test_swift_failure_raises(tmp_path):
    d = np.load(os.path.join(GOLD, "encounters_t50.npz"))
    bad = tmp_path / "swift_fail"
    bad.write_text("#!/bin/sh\nexit 3\n")
    bad.chmod(0o755)
    sim, _ = make_sim(d, tmp_path, str(bad))
    sim.init()
    with pytest.raises(G.GlisserError, match="swift did not terminate normally"):
        for _ in range(int(d["nblocks"])):
            sim.loop()


def test_missing_swift_program_raises(tmp_path):
    d = np.load(os.path.join(GOLD, "encounters_t50.npz"))
    sim, _ = make_sim(d, tmp_path, str(tmp_path / "no_such_program"))
    sim.init()
    with pytest.raises(G.GlisserError, match="Swift-Path"):
        for _ in range(int(d["nblocks"])):
            sim.loop()


def test_run_writes_stat_and_timing(tmp_path, monkeypatch):
    """glisser_run with Resolve-Encounters: stat.out and timing.out in the
    output folder, and a state.out that matches the stepped run's."""
    d = np.load(os.path.join(GOLD, "encounters_t50.npz"))
    swift = fake_swift.wrapper(str(tmp_path))
    monkeypatch.delenv("FAKE_SWIFT_ARCHIVE", raising=False)
    cfgfile = tmp_path / "run"
    cfgfile.mkdir()
    plh = os.path.join(GOLD, "plhist_yr.bin")
    state = tmp_path / "state.in"
    pl_m, pl_r, pl_v = d["pl_m"], d["pl_r"], d["pl_v"]
    with open(state, "w") as f:
        f.write("%d\n" % len(pl_m))
        for i in range(len(pl_m)):
            f.write("%.17g\n%.17g %.17g %.17g\n%.17g %.17g %.17g\n%d\n" % (pl_m[i], *pl_r[i], *pl_v[i], i))
        f.write("%d\n" % len(d["r0"]))
        for k in range(len(d["r0"])):
            f.write("%.17g %.17g %.17g\n%.17g %.17g %.17g\n%d 0 0\n" % (*d["r0"][k], *d["v0"][k], d["id0"][k]))
    tf = float(d["counts"][-1][0])
    cfg = (str(d["config"]).replace("Final-Time 1e9", "Final-Time %r" % tf) +
           "\nPlanet-History-File %s\nSwift-Path %s\nOutput-Folder %s\nInput-File %s\n" % (plh, swift, cfgfile, state))
    run = G.Simulation(cfg)
    run.run(quiet=True, force=True)
    assert (cfgfile / "stat.out").exists() and (cfgfile / "timing.out").exists()
    timing = open(cfgfile / "timing.out").read().strip().split("\n")
    assert timing[0].startswith("t,") and len(timing) == 1 + int(d["nblocks"])
    ours = parse_stat(open(cfgfile / "stat.out").read())
    assert sorted(ours) == sorted(parse_stat(str(d["stat_out"])))
    enc = parse_log(open(cfgfile / "encounter.out").read())
    assert enc == parse_log(str(d["encounter_log"]))
