"""The targets/main.cpp driver as a library call (glisser_run): output
folder layout, track snapshots (device writer), dumps written by the writer
thread, planetary history, end state -- against a block-by-block run of the
same input through the executor."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import glisser_gb300 as G  # noqa: E402
from glisser_gb300 import synth  # noqa: E402
from glisser_gb300.shard import read_track  # noqa: E402
from test_gpu_track import same_records  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def native():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    G.build()
    G.lib()


def test_run_writes_reference_layout_and_matches_block_loop(tmp_path):
    m, pr, pv, r, v = synth.cartesian_state("plain-neptune", 3000, seed=41)
    base = "Time-Step 180\nTime-Block-Size 64\nCull-Radius 0.5\n"
    pre = G.Simulation(base + "Input-File unused\nOutput-Folder unused\n")
    pre.set_planets(m, pr, pv)
    pre.set_particles(r, v)
    state = str(tmp_path / "state.in")
    pre.write_state(state)
    out = str(tmp_path / "out")
    cfg = (base + "Final-Time %r\nTrack-Interval 2\nDump-Interval 3\nSwift-History-Interval 2\nLog-Interval 1\n"
           "Input-File %s\nOutput-Folder %s\n" % (6 * 64 * 180.0, state, out))
    run = G.Simulation(cfg)
    run.load_state()
    run.run(quiet=True, force=True)
    for f in ("config.in", "state.in", "stdout", "encounter.out", "time.out", "state.out", "config.out",
              "plhist.out", "tracks/track.0.out", "dumps/state.0.out", "dumps/config.0.out", "dumps/state.1.out",
              "dumps/config.1.out"):
        assert os.path.exists(os.path.join(out, f)), f
    snaps = read_track(os.path.join(out, "tracks/track.0.out"))
    assert len(snaps) == 4                                  # start + every 2 of 6 blocks

    # the same input block by block
    ref = G.Simulation(base + "Input-File %s\nOutput-Folder unused\n" % state)
    ref.load_state()
    ref.init()
    for b in range(6):
        ref.loop()
        if b == 2:
            dump3 = ref.particles()
    final = ref.particles()
    back = G.Simulation("Input-File %s\nOutput-Folder unused\n" % os.path.join(out, "state.out"))
    back.load_state()
    got = back.particles()
    o, q = np.argsort(got["id"]), np.argsort(final["id"])
    assert np.array_equal(got["id"][o], final["id"][q])
    assert np.array_equal(got["flags"][o], final["flags"][q])
    assert np.array_equal(got["r"][o], final["r"][q]) and np.array_equal(got["v"][o], final["v"][q])
    # the dump is written in the run's output format (ASCII here) although its
    # config.N.out says binary output -- the reference's behaviour
    # (targets/main.cpp:208-225: save_data with the run configuration)
    assert "Write-Binary-Output 1" in open(os.path.join(out, "dumps/config.0.out")).read()
    d0 = G.Simulation("Input-File %s\nOutput-Folder unused\n" % os.path.join(out, "dumps/state.0.out"))
    d0.load_state()
    dd = d0.particles()
    o, q = np.argsort(dd["id"]), np.argsort(dump3["id"])
    assert np.array_equal(dd["r"][o], dump3["r"][q])

    # last snapshot against the host writer on the block-by-block run
    p = str(tmp_path / "host.track")
    ref.set_device_output(False)
    ref.write_track(p)
    h = read_track(p)[0]
    assert h[0] == snaps[-1][0] and h[1].tobytes() == snaps[-1][1].tobytes()
    same_records(snaps[-1][2], h[2])


def test_resume_from_dump_matches_uninterrupted_run(tmp_path):
    """Checkpoint / resume: a run restarted from its first dump (the dump's
    configuration with Input-File pointed at the dump state) reaches the same
    end state as the uninterrupted run -- same flags and survivors, positions
    within 1e-12 (the restart recomputes the carried accelerations on the
    host, as the reference's init does)."""
    m, pr, pv, r, v = synth.cartesian_state("plain-neptune", 2000, seed=43)
    base = "Time-Step 180\nTime-Block-Size 64\nCull-Radius 0.5\n"
    pre = G.Simulation(base + "Input-File unused\nOutput-Folder unused\n")
    pre.set_planets(m, pr, pv)
    pre.set_particles(r, v)
    state = str(tmp_path / "state.in")
    pre.write_state(state)
    tf = 8 * 64 * 180.0
    out = str(tmp_path / "full")
    full = G.Simulation(base + "Final-Time %r\nDump-Interval 3\nInput-File %s\nOutput-Folder %s\n" % (tf, state, out))
    full.load_state()
    full.run(quiet=True, force=True)

    lines = open(os.path.join(out, "dumps/config.0.out")).read().splitlines()
    keep = [l for l in lines if l.split(" ", 1)[0] not in ("Input-File", "Output-Folder", "Final-Time",
                                                            "Read-Binary-Input", "Write-Binary-Output")]
    out2 = str(tmp_path / "resumed")
    cfg2 = "\n".join(keep + ["Final-Time %r" % tf, "Input-File %s" % os.path.join(out, "dumps/state.0.out"),
                             "Output-Folder %s" % out2]) + "\n"
    res = G.Simulation(cfg2)
    res.load_state()
    res.run(quiet=True, force=True)

    a = G.Simulation("Input-File %s\nOutput-Folder unused\n" % os.path.join(out, "state.out"))
    a.load_state()
    b = G.Simulation("Input-File %s\nOutput-Folder unused\n" % os.path.join(out2, "state.out"))
    b.load_state()
    pa, pb = a.particles(), b.particles()
    oa, ob = np.argsort(pa["id"]), np.argsort(pb["id"])
    assert np.array_equal(pa["id"][oa], pb["id"][ob])
    assert np.array_equal(pa["flags"][oa], pb["flags"][ob])
    live = pa["flags"][oa] == 0
    err = np.linalg.norm(pa["r"][oa] - pb["r"][ob], axis=1) / np.linalg.norm(pa["r"][oa], axis=1)
    assert err[live].max() < 1e-12
    np.testing.assert_allclose(a.planets()["r"], b.planets()["r"], rtol=1e-12, atol=1e-12)
