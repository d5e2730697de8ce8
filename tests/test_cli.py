"""The glisser command (targets/main.cpp:29-60 over glisser_run): usage,
configuration errors reported as the reference reports them, refusal of a
non-empty output folder without --force; on the GPU, a whole run writes the
reference's output folder layout, from the executable and from
`python -m glisser_gb300`."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import glisser_gb300 as G  # noqa: E402

EXE = os.path.join(os.path.dirname(G.LIB_PATH), "glisser")


@pytest.fixture(scope="module", autouse=True)
def built():
    G.build()


def run(args, cwd):
    return subprocess.run([EXE] + args, capture_output=True, text=True, cwd=cwd, timeout=600)


def test_usage_and_bad_arguments(tmp_path):
    r = run(["--help"], tmp_path)
    assert r.returncode == 0 and "glisser [options] [<config>]" in r.stdout
    r = run(["--no-such-option"], tmp_path)
    assert r.returncode == 1 and "Usage:" in r.stderr


def test_missing_and_invalid_configuration(tmp_path):
    r = run([], tmp_path)                                   # config.in by default, absent
    assert r.returncode == 255 and "Reading from configuration file config.in" in r.stdout
    assert "Could not read configuration." in r.stderr
    (tmp_path / "bad.in").write_text("Time-Step abc\n")
    r = run(["bad.in"], tmp_path)
    assert r.returncode == 255 and "Could not read configuration." in r.stderr


def small_run(tmp_path):
    from glisser_gb300 import synth
    m, pr, pv, r, v = synth.cartesian_state("plain-neptune", 500, seed=3)
    pre = G.Simulation("Time-Step 180\nTime-Block-Size 64\nInput-File unused\nOutput-Folder unused\n")
    pre.set_planets(m, pr, pv)
    pre.set_particles(r, v)
    pre.write_state(str(tmp_path / "state.in"))
    cfg = ("Time-Step 180\nTime-Block-Size 64\nFinal-Time %r\nTrack-Interval 1\nDump-Interval 2\nLog-Interval 1\n"
           "Input-File state.in\nOutput-Folder out\n" % (4 * 64 * 180.0))
    (tmp_path / "config.in").write_text(cfg)


@pytest.mark.gpu
def test_command_writes_the_reference_layout(tmp_path):
    small_run(tmp_path)
    r = run([], tmp_path)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "out"
    for f in ("config.in", "state.in", "stdout", "encounter.out", "time.out", "state.out", "config.out",
              "tracks/track.0.out", "dumps/state.0.out", "dumps/config.0.out"):
        assert (out / f).exists(), f
    assert "Host uses little-endian doubles? yes" in r.stdout
    r = run([], tmp_path)                                   # non-empty output folder, no --force
    assert r.returncode == 255 and "not empty" in r.stderr
    r = run(["--force", "--quiet", "config.in"], tmp_path)
    assert r.returncode == 0 and "little-endian" not in r.stdout
    # the Python front-end gives the same end state
    r2 = subprocess.run([sys.executable, "-m", "glisser_gb300", "--force", "--quiet", "config.in"], cwd=tmp_path,
                        capture_output=True, text=True, timeout=600, env=dict(os.environ, PYTHONPATH=ROOT))
    assert r2.returncode == 0, r2.stderr
    a = G.Simulation("Input-File %s\nOutput-Folder unused\n" % (out / "state.out"))
    a.load_state()
    p = a.particles()
    assert len(p["id"]) == 500 and np.isfinite(p["r"]).all()
