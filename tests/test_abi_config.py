"""C ABI surface and configuration parity (CPU only: no call here needs a GPU).

* the native library loads and exports every entry point include/glisser.h
  declares;
* configuration texts are accepted or rejected with the reference's messages
  (read_configuration, src/data.cpp:195-333; fixture from the reference);
* the written configuration matches write_configuration byte for byte,
  including its Encounter-RH-Factor quirk (src/data.cpp:342).
"""
import ast
import os
import re

import pytest

import glisser_gb300 as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module", autouse=True)
def native():
    G.build()
    G.lib()


def header_symbols():
    text = open(os.path.join(ROOT, "include", "glisser.h")).read()
    return sorted(set(re.findall(r"\b(glisser_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    import ctypes
    L = ctypes.CDLL(G.LIB_PATH)
    names = header_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_config_errors_match_reference():
    for line in open(os.path.join(GOLD, "config_errors.txt")):
        text_repr, rc, msg = line.rstrip("\n").split("\t")
        text = ast.literal_eval(text_repr)
        with pytest.raises(G.ConfigError) as ei:
            G.Simulation(text)
        assert msg in str(ei.value)


def test_config_written_matches_reference(tmp_path):
    text = open(os.path.join(GOLD, "config_in.txt")).read()
    sim = G.Simulation(text)
    out = tmp_path / "config.out"
    sim.write_config(str(out), float(sim.config("Initial-Time")), float(sim.config("Final-Time")))
    assert out.read_text() == open(os.path.join(GOLD, "config_written.txt")).read()


def test_config_defaults_and_keys():
    sim = G.Simulation("Input-File x\n")
    assert sim.config("Time-Block-Size") == "1024"
    assert sim.config("Outer-Limit") == "300"
    assert sim.config("Cull-Radius") == "0.5"
    assert sim.config("Output-Folder") == "output/"
    assert sim.config("Limit-Particle-Count") == "4294967295"
    sim = G.Simulation("# comment\n\nTime-Step 0.25\nBig-G 2\nInput-File y\nRead-Planet-History 1\n"
                       "Planet-History-File h.bin\nResolve-Encounters 1\n")
    assert sim.config("Time-Step") == "0.25"
    assert sim.config("Big-G") == "2"
    assert sim.config("Resolve-Encounters") == "1"


def test_calls_before_init_fail_cleanly():
    sim = G.Simulation("Input-File x\n")
    with pytest.raises(G.GlisserError):
        sim.init()            # no state loaded
    with pytest.raises(G.GlisserError):
        sim.loop()
    with pytest.raises(G.GlisserError) as ei:
        sim.load_state()      # missing input file
    assert ei.value.code == G.E_IO
