"""File formats and the host planet producer against the reference's own
outputs (tests/golden, written by the unmodified reference).  CPU only: the
executor runs planets-only (no particles) without touching a GPU, and the
writers work on the loaded state.
"""
import os
import platform

import numpy as np
import pytest

import glisser_gb300 as G

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EXACT_HOST = platform.machine() in ("x86_64", "AMD64")


@pytest.fixture(scope="module", autouse=True)
def native():
    G.build()
    G.lib()


def close(x, y, rel=1e-13):
    x = np.asarray(x, np.float64); y = np.asarray(y, np.float64)
    if EXACT_HOST:
        return np.array_equal(x, y)
    return bool(np.all(np.abs(x - y) <= rel * np.maximum(np.abs(y), 1e-300)))


def test_element_conversions():
    g = np.load(os.path.join(GOLD, "elements.npz"))
    mu = float(g["mu"])
    r, v = G.elements_to_cartesian(mu, g["el"])
    np.testing.assert_allclose(r, g["r"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(v, g["v"], rtol=1e-12, atol=1e-15)
    for k in range(0, len(r), 5):
        es, back = G.to_elements(mu, g["r"][k], g["v"][k])
        assert es == g["esign"][k]
        np.testing.assert_allclose(back, g["back"][k], rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("case", ["neptune_t128", "giants_t256", "interp_t50"])
def test_planet_blocks_match_reference(case):
    """Planet log, h0 log, masses, ids and encounter radii per block."""
    d = np.load(os.path.join(GOLD, case + ".npz"))
    cfg = str(d["config"]).replace("Planet-History-File ", "#")
    extra = "\nInput-File unused\nOutput-Folder unused\nLimit-Particle-Count 0\n"
    if "Read-Planet-History 1" in cfg:
        extra += "Planet-History-File %s\n" % os.path.join(GOLD, "plhist_yr.bin")
    sim = G.Simulation(cfg + extra)
    sim.set_planets(d["pl_m"], d["pl_r"], d["pl_v"], np.arange(len(d["pl_m"])))
    sim.set_particles(np.zeros((0, 3)), np.zeros((0, 3)))
    sim.init()
    for b in range(int(d["nblocks"])):
        blk = sim.planet_block()
        want_r = d["blk%d_r_log" % b]
        assert close(blk["r_log"], want_r), b
        assert close(blk["h0_log"], d["blk%d_h0_log" % b]), b
        assert close(blk["m"], d["blk%d_m" % b]) and close(blk["rh"], d["blk%d_rh" % b])
        assert np.array_equal(blk["id"], d["blk%d_id" % b])
        sim.loop()
    pl = sim.planets()
    assert close(pl["r"], d["final_pl_r"]) and close(pl["v"], d["final_pl_v"])


def test_planets_only_preintegration_writes_reference_history(tmp_path):
    """Planets-only run (Limit-Particle-Count 0) writing a planetary history
    every 20 blocks: the file the reference wrote for the same run."""
    d = np.load(os.path.join(GOLD, "interp_t50.npz"))
    sim = G.Simulation("Time-Step 0.2\nTime-Block-Size 5\nFinal-Time 1e9\nLimit-Particle-Count 0\n"
                       "Input-File unused\nOutput-Folder unused\n")
    sim.set_planets(d["pl_m"], d["pl_r"], d["pl_v"], np.arange(3))
    sim.set_particles(np.zeros((0, 3)), np.zeros((0, 3)))
    sim.init()
    path = str(tmp_path / "plhist.out")
    sim.write_plhist(path, begin=True)
    for b in range(800):
        sim.loop()
        if (b + 1) % 20 == 0:
            sim.write_plhist(path)
    got = open(path, "rb").read()
    want = open(os.path.join(GOLD, "plhist_yr.bin"), "rb").read()
    assert len(got) == len(want)
    if EXACT_HOST:
        assert got == want
    else:
        a = np.frombuffer(got, np.uint8); b = np.frombuffer(want, np.uint8)
        assert (a != b).mean() < 0.01


def _formats_state():
    d = np.load(os.path.join(GOLD, "formats_run.npz"))
    b = int(d["nblocks"]) - 1
    return d, b


def test_state_files_byte_identical(tmp_path):
    d, b = _formats_state()
    sim = G.Simulation("Initial-Time %r\nInput-File unused\nOutput-Folder unused\n" % float(d["out%d_t" % b]))
    sim.set_planets(d["final_pl_m"], d["final_pl_r"], d["final_pl_v"], d["final_pl_id"])
    sim.set_particles(d["out%d_r" % b], d["out%d_v" % b], d["out%d_id" % b], d["out%d_flags" % b],
                      d["out%d_deathtime" % b])
    for binary, name in ((False, "state_ascii.out"), (True, "state_binary.out")):
        p = str(tmp_path / name)
        sim.write_state(p, binary=binary)
        assert open(p, "rb").read() == open(os.path.join(GOLD, name), "rb").read(), name


def test_state_round_trip(tmp_path):
    d, b = _formats_state()
    for binary in (False, True):
        p = str(tmp_path / ("s.bin" if binary else "s.txt"))
        sim = G.Simulation("Input-File unused\nOutput-Folder unused\n")
        sim.set_planets(d["final_pl_m"], d["final_pl_r"], d["final_pl_v"], d["final_pl_id"])
        sim.set_particles(d["out%d_r" % b], d["out%d_v" % b], d["out%d_id" % b], d["out%d_flags" % b],
                          d["out%d_deathtime" % b])
        sim.write_state(p, binary=binary)
        back = G.Simulation("Input-File %s\nRead-Binary-Input %d\nOutput-Folder unused\n" % (p, int(binary)))
        back.load_state()
        pa = back.particles()
        assert np.array_equal(pa["r"], d["out%d_r" % b]) and np.array_equal(pa["v"], d["out%d_v" % b])
        assert np.array_equal(pa["id"], d["out%d_id" % b]) and np.array_equal(pa["flags"], d["out%d_flags" % b])
        assert np.array_equal(pa["deathtime"], d["out%d_deathtime" % b])
        pl = back.planets()
        assert np.array_equal(pl["m"], d["final_pl_m"]) and np.array_equal(pl["r"], d["final_pl_r"])


@pytest.mark.parametrize("bary,name", [(1, "track_bary.out"), (0, "track_helio.out")])
def test_track_file(tmp_path, bary, name):
    d, b = _formats_state()
    alive = d["out%d_flags" % b] == 0
    sim = G.Simulation("Initial-Time %r\nWrite-Barycentric-Track %d\nInput-File unused\nOutput-Folder unused\n"
                       % (float(d["out%d_t" % b]), bary))
    sim.set_planets(d["final_pl_m"], d["final_pl_r"], d["final_pl_v"], d["final_pl_id"])
    sim.set_particles(d["out%d_r" % b][alive], d["out%d_v" % b][alive], d["out%d_id" % b][alive])
    p = str(tmp_path / name)
    sim.write_track(p)
    got = open(p, "rb").read()
    want = open(os.path.join(GOLD, name), "rb").read()
    assert len(got) == len(want)
    if got != want:
        # float32 elements may differ in the last place where libm does
        ga = np.frombuffer(got[16:], np.uint8); wa = np.frombuffer(want[16:], np.uint8)
        assert (ga != wa).mean() < 0.02


def test_plhist_record(tmp_path):
    d, b = _formats_state()
    sim = G.Simulation("Initial-Time %r\nInput-File unused\nOutput-Folder unused\n" % float(d["out%d_t" % b]))
    sim.set_planets(d["final_pl_m"], d["final_pl_r"], d["final_pl_v"], d["final_pl_id"])
    sim.set_particles(np.zeros((0, 3)), np.zeros((0, 3)))
    p = str(tmp_path / "plhist.out")
    sim.write_plhist(p, begin=True)
    assert open(p, "rb").read() == open(os.path.join(GOLD, "plhist_fmt.out"), "rb").read()
