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


@pytest.mark.parametrize("kernel", sorted(bench.FP64_COUNTS))
def test_executed_fp64_view(kernel):
    v = bench.executed_fp64(kernel, 1e10, 1.25)
    c = bench.FP64_COUNTS[kernel]
    flops = c["dadd"] + c["dmul"] + 2 * c["dfma"]
    assert v["flops_per_particle_step"] == pytest.approx(flops)
    assert v["achieved"] == pytest.approx(1e10 * flops / 1e12)
    assert v["frac"] == pytest.approx(v["achieved"] / 1.25)
    assert 0 < v["fp64_pipe_busy"] <= 1
    assert os.path.exists(os.path.join(ROOT, c["profile"]))
    assert bench.executed_fp64("no such kernel", 1e10, 1.25) is None


def test_reference_arm_does_not_load_the_library():
    """The reference arm times the reference's CPU code on inputs the oracle
    makes: this library's shared object is never mapped."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', "
            "'--sample-particles', '256', '--sample-steps', '8']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); print('LOADED' if 'libglisser_gb300' in maps else 'CLEAN')")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip().splitlines()[-1] == "CLEAN"


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
