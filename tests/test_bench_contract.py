"""The benchmark's JSON contract on the CPU: the reference arm (the oracle's
restatement of the reference kernel on the host cores) prints one line with
the keys the contract names, and the roofline helpers follow the fixed
algorithmic-flop convention."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_algorithmic_flops_convention():
    # F = 99 + 14 K + 18 Np with K = 5 Newton passes of the reference formulation
    assert bench.alg_flops_per_particle_step(4) == 241
    assert bench.alg_flops_per_particle_step(1) == 187
    assert bench.alg_flops_per_particle_step(4, k_ref=3) == 213


def test_executed_fp64_view():
    v = bench.executed_fp64_view(4, 1e10, 1.25)
    c = bench.FP64_INSTR_PER_STEP_NP4
    flops = c["dadd"] + c["dmul"] + 2 * c["dfma"]
    assert v["flops_per_particle_step"] == pytest.approx(flops)
    assert v["achieved"] == pytest.approx(1e10 * flops / 1e12)
    assert v["frac"] == pytest.approx(v["achieved"] / 1.25)
    assert 0 < v["fp64_pipe_busy"] <= 1
    assert bench.executed_fp64_view(1, 1e10, 1.25) is None     # counted for the 4-planet kernel only


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1", "--sample-particles", "1024", "--sample-steps", "32"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "particle-steps/s"
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert "workload" in d["config"]
