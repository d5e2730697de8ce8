"""Benchmark: particle-steps/s of the massless-particle WH/MVS time-block
integrator on GB300, learned starter + batching against the plain kernel.

Headline workload (`value`): the batched-ensembles workload -- 256 independent
systems, each the Sun + four giant planets with masses x U(0.9, 1.1) and
semi-major axes x U(0.95, 1.05), lognormal particle counts (median 2e4,
clipped to 1e3..2e5, ~6.15e6 particles in all) with a~U(40,50) au, e<0.1,
i<5 deg; FP64, dt = 180 d -- run by the learned starter in the persistent,
graph-captured batched kernel with the autotuned launch shape.  One bench step
= one time block of every system.  `value` is device-resident throughput over
K blocks timed with CUDA events on the ensemble's stream; `e2e` repeats blocks
through the public API with host buffers (every particle's state uploaded
before and downloaded after each block inside the timed region).

Beside it, on the same workload: the plain kernel (the single-system
time-block kernel with the series starter, one system per launch -- how a
kernel without batching runs an ensemble) and the reference's own method (its
classic starter) the same way, the batched kernel with the series starter,
and an accuracy check of the batched legs against the FP64 oracle.  Other
legs: the plain-giants workload (1e6 particles, T = 2048) with the
float-float and the FP64 planet kick and the reference's own GPU kernel on the
same block, the scattered disk, the close-eccentric regime where the learned
starter runs its network, the planetary-history + encounter-flagging
workload, and the track/dump streams.

`roofline` relates the batched kernel's executed FP64 flops (instruction
counts of this build from ncu, per particle-step) to the FP64 FMA throughput
the library's probe measures on the same GPU.  `cpu_baseline` times the
reference's own CPU build of its kernel arithmetic (MVSKernel::step_forward,
src/wh.cu:113-177) on a sample of the headline workload on the host cores.
`--impl reference` times that CPU implementation as the reference arm without
loading this library.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300, learned+batched vs plain, at <=1e-10 rel pos err"
UNIT = "particle-steps/s"
KEPLER_TOL_SCATTERED = 1e-14     # the scattered-disk workload's Newton tolerance
ENSEMBLE_WORKLOAD = ("ensembles: 256 systems (Sun + 4 giants, masses x U(0.9,1.1), a x U(0.95,1.05)), lognormal "
                     "particle counts (median 2e4, clipped 1e3..2e5), particles a~U(40,50) au e~U(0,0.1) "
                     "i~U(0,5deg), FP64, dt=180 d")

# Executed FP64 thread-instructions per particle-step counted by ncu
# (smsp__sass_thread_inst_executed_op_d{add,fma,mul}_pred_on.sum over one
# launch, divided by the launch's particle-steps) and the FP64 pipe's busy
# share (sm__pipe_fp64_cycles_active, pct of peak sustained active), for the
# kernels whose rooflines the bench reports; the captures and their commands
# are summarised under profiles/.
FP64_COUNTS = {
    "batched_kernel<4,128,1,series>": {"dadd": 1.0, "dfma": 26.0, "dmul": 17.0, "pipe_busy": 0.776,
                                       "profile": "profiles/batched_kernel_ensembles.md"},
    "timeblock_kernel<4>": {"dadd": 1.0, "dfma": 26.0, "dmul": 17.0, "pipe_busy": 0.709,
                            "profile": "profiles/timeblock_kernel_plain-giants.md"},
}
# DRAM bytes per particle per block of the batched kernel (ncu dram__bytes_read
# + dram__bytes_write, 153.2 + 78.8 MB, on a capture of one block of a quarter
# of the headline workload: 1,537,972 particles, T = 1024)
DRAM_BYTES_PER_PARTICLE_BLOCK = 150.8


def alg_flops_per_particle_step(n_planets, k_ref=5):
    """Algorithmic FP64 flops per particle-step (reference formulation):
    2 kicks 12, drift prelude 45, K Newton passes 14 each, f/g and the new
    state 37, 18 per planet, 5 for the Sun/outer tests."""
    return 99 + 14 * k_ref + 18 * n_planets


def executed_fp64(kernel, rate, peak_tf):
    """FP64 flops the named kernel executes (DADD + DMUL + 2 DFMA per
    particle-step, ncu counts) at `rate` particle-steps/s, against the probe
    peak.  A DADD or DMUL fills an FP64 issue slot with one flop, so `frac`
    counts flops and `fp64_pipe_busy` the slots."""
    key = kernel if kernel in FP64_COUNTS else None
    if key is None:
        # per-thread instruction counts do not depend on the CTA size
        key = next((k for k in FP64_COUNTS if k.split(",")[0] == kernel.split(",")[0] and
                    k.split(",")[2:] == kernel.split(",")[2:]), None)
    c = FP64_COUNTS.get(key)
    if c is None or not rate:
        return None
    flops = c["dadd"] + c["dmul"] + 2 * c["dfma"]
    tf = rate * flops / 1e12
    return {"kernel": kernel, "counts_from": key,
            "instructions_per_particle_step": round(c["dadd"] + c["dmul"] + c["dfma"], 1),
            "flops_per_particle_step": flops, "achieved": tf, "peak": peak_tf, "unit": "TFLOP/s",
            "frac": tf / peak_tf if peak_tf else None, "fp64_pipe_busy": c["pipe_busy"], "source": c["profile"]}


def config_text(tbsize, dt, outer=300.0, extra=""):
    return ("Time-Step %r\nTime-Block-Size %d\nFinal-Time 1e30\nOuter-Limit %r\nCull-Radius 0.5\n%s"
            "Input-File unused\nOutput-Folder unused\n" % (dt, tbsize, outer, extra))


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# Workloads


def ensemble_elements(rank, fraction=1.0, n_systems=256):
    """Per system (masses, planet elements, particle elements) of the headline
    workload; seeds depend on the rank (independent shards per GPU)."""
    from glisser_gb300 import synth
    return synth.ensemble_workload(n_systems, seed=1000 * rank, fraction=fraction)


def to_cartesian(conv, systems):
    """(masses, planet r, planet v, particle r, particle v) per system, with
    `conv(mu, elements) -> r, v` (the library's, or the oracle's where the
    library must not be loaded)."""
    out = []
    for m, pel, el in systems:
        pr, pv = [np.zeros(3)], [np.zeros(3)]
        for k in range(len(m) - 1):
            a, b = conv(m[0] + m[k + 1], pel[k:k + 1])
            pr.append(a[0])
            pv.append(b[0])
        r, v = conv(m[0], el)
        out.append((m, np.array(pr), np.array(pv), r, v))
    return out


def perihelion_below(m, r, v, q_max):
    """Particles whose osculating perihelion is below q_max."""
    mu = m[0]
    r0 = np.linalg.norm(r, axis=1)
    a = 1.0 / (2.0 / r0 - (v * v).sum(1) / mu)
    h = np.cross(r, v)
    e = np.sqrt(np.maximum(0.0, 1.0 - (h * h).sum(1) / (mu * a)))
    return (a > 0) & (a * (1 - e) < q_max)


# ---------------------------------------------------------------------------
# CPU baseline and the reference arm (no product library on this path)


def reference_cpu_rate(systems, sample_particles, sample_steps, threads, dt=180.0, outer=300.0):
    """The reference's own host build of MVSKernel::step_forward
    (src/wh.cu:113-177; oracle/_ref) -- or, where it was not built, the
    oracle's restatement of it -- over a sample of the workload: the first
    systems' particles up to `sample_particles`, `sample_steps` steps of each
    system's planet block (the oracle's planet integrator), split across host
    threads (ctypes releases the GIL).  Returns (rate, seconds, kind)."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    kind = "reference" if O.reference_lib() is not None else "port"
    jobs = []
    left = sample_particles
    for m, pr, pv, r, v in systems:
        if left <= 0:
            break
        k = min(left, len(r))
        left -= k
        ex = O.Exec(m, pr, pv, np.arange(len(m)), r[:k], v[:k], np.arange(k), dt=dt, tbsize=sample_steps,
                    outer_r=outer)
        p = ex.particles()
        blk = ex.planet_block()
        for idx in np.array_split(np.arange(k), max(1, min(threads, (k + 511) // 512))):
            jobs.append((p["r"][idx].copy(), p["v"][idx].copy(), p["a"][idx].copy(), blk))
    n_total = sum(len(j[0]) for j in jobs)

    def work(job):
        r, v, a, blk = job
        npl = len(blk["m"])
        args = (r, v, a, np.zeros(len(r), np.uint16), sample_steps, npl, blk["h0_log"], blk["r_log"], blk["m"],
                blk["id"], blk["rh"], outer, dt, float(blk["m"][0]))
        if kind == "reference":
            O.reference_block(*args)
        else:
            O.block(*args, drift="mvs")
        return len(r)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as pool:
        done = sum(pool.map(work, jobs))
    el = time.perf_counter() - t0
    assert done == n_total
    return n_total * sample_steps / el, el, kind


def cpu_sample_note(kind, n, steps, threads):
    what = ("the reference's own MVSKernel::step_forward (src/wh.cu:113-177) compiled for the host from its "
            "sources (oracle/_ref)" if kind == "reference" else
            "the oracle's restatement of MVSKernel::step_forward (src/wh.cu:113-177)")
    return ("%s on %d particles of the first systems x %d steps per step, %d host threads; per-particle-step rate "
            "extrapolated to the whole workload" % (what, n, steps, threads))


def run_reference_arm(args, rank, world):
    """The reference's CPU implementation of the path on the host cores, on the
    headline workload's distributions: same metric, config and unit as the GPU
    arm.  Inputs come from the oracle's element conversion; this library is
    not loaded."""
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    systems = to_cartesian(O.elements_to_cartesian, ensemble_elements(0, fraction=args.ensemble_fraction))
    threads = os.cpu_count() or 1
    kind = None
    # each step a quarter of the GPU arm's CPU sample (~1.7 s on 16 cores), so
    # that --steps 20 --warmup 5 ends within a minute or so
    sample = max(1, args.sample_particles // 4)
    for _ in range(args.warmup):
        reference_cpu_rate(systems, sample, args.sample_steps, threads)
    els = []
    for _ in range(args.steps):
        _, el, kind = reference_cpu_rate(systems, sample, args.sample_steps, threads)
        els.append(el)
    value = len(els) * sample * args.sample_steps / sum(els)
    note = cpu_sample_note(kind, sample, args.sample_steps, threads)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(els) / len(els), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": ENSEMBLE_WORKLOAD, "systems": 256, "n_planets": 4, "l2": "n/a (host CPU)",
                   "sample": note},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": note},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# The learned starter


def train_starter(G, args, rank):
    """A network for the learned starter, trained on the plain method's Kepler
    solves logged from the scattered disk's pericentre passages -- the drifts
    with tau^2 = dt^2 mu / r^3 >= the log floor, where the kernels run the
    network (elsewhere the series starter runs): the particles with perihelion
    below 12 au, logged every 16 steps."""
    from glisser_gb300 import learned as L
    from glisser_gb300 import synth
    m, pr, pv, r, v = synth.cartesian_state("scattered-disk", args.learned_particles, seed=2000 + rank)
    sel = perihelion_below(m, r, v, 12.0)
    sim = G.Simulation(config_text(16, 180.0, outer=1e5))
    sim.set_planets(m, pr, pv)
    sim.set_particles(r[sel], v[sel])
    sim.init()
    tr = L.Trainer(int(sel.sum()) * args.learned_log_blocks + 1, seed=7)
    tr.set_log_floor(L.LOG_TAU2_FLOOR)
    logged = 0
    t0 = time.perf_counter()
    for _ in range(args.learned_log_blocks):
        logged += sim.counts()["n_alive"]
        tr.log_simulation(sim)
        sim.loop()
    t_log = time.perf_counter() - t0
    del sim
    n_kept, evals = tr.samples()
    tr.fit_norm()
    t0 = time.perf_counter()
    losses = tr.train(args.learned_train_steps, batch=16384, lr=3e-3, lr_min=1e-5, seed=11)
    t_train = time.perf_counter() - t0
    path = os.path.join(tempfile.mkdtemp(), "starter.bin")
    tr.save(path)
    info = {"solves_logged": logged, "kept_tau2_floor": n_kept, "tau2_floor": L.LOG_TAU2_FLOOR,
            "plain_evals_per_kept_solve": evals / max(n_kept, 1), "log_s": t_log, "train_s": t_train,
            "steps": args.learned_train_steps, "batch": 16384, "loss_first": float(losses[:10].mean()),
            "loss_last": float(losses[-100:].mean()), "network": "3-32-32-1 SiLU, BF16 weights, FP32 accumulate",
            "logged_from": "scattered-disk particles with perihelion < 12 au (%d of %d), every 16 steps"
                           % (int(sel.sum()), len(r))}
    return path, tr, info


# ---------------------------------------------------------------------------
# Headline: the batched ensembles


def make_ensemble(G, systems, T, starter, path=None, shape=None):
    ens = G.Ensemble(config_text(T, 180.0), len(systems))
    for s, (m, pr, pv, r, v) in enumerate(systems):
        ens.set_system(s, m, pr, pv, r, v)
    ens.set_starter(starter, path)
    if shape:
        ens.set_shape(*shape)
    ens.init()
    return ens


def time_ensemble(ens, steps, warmup, barrier, clocks=None, flush=None):
    """W warm-up blocks, then `steps` blocks timed with CUDA events on the
    ensemble's stream (max over ranks by the caller)."""
    import torch
    stream = torch.cuda.ExternalStream(ens.stream())
    for _ in range(warmup):
        ens.step()
    barrier()
    if clocks:
        clocks.start()
    s0 = ens.stats()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    kms = []
    for _ in range(steps):
        kms.append(ens.step())
    e1.record(stream)
    e1.synchronize()
    barrier()
    clk = clocks.stop() if clocks else None
    s1 = ens.stats()
    d = {k: s1[k] - s0[k] for k in s0}
    return e0.elapsed_time(e1), kms, d, clk


def plain_one_at_a_time(G, systems, T, starter, n_systems):
    """The single-system kernel over the workload one system per launch (a
    Simulation per system, one warm-up block, one timed block each): how a
    kernel without batching runs an ensemble."""
    ps, el = 0, 0.0
    for m, pr, pv, r, v in systems[:n_systems]:
        sim = G.Simulation(config_text(T, 180.0))
        sim.set_planets(m, pr, pv)
        sim.set_particles(r, v)
        sim.set_starter(starter)
        sim.init()
        sim.loop()
        a = sim.stats()["particle_steps"]
        t0 = time.perf_counter()
        sim.loop()
        el += time.perf_counter() - t0
        ps += sim.stats()["particle_steps"] - a
        del sim
    return ps / el


def ensemble_vs_oracle(G, path, T=256, blocks=4, n_systems=8, n_particles=512):
    """The batched kernel (series and learned starters) against the oracle's
    block loop (the reference kernel's arithmetic and planet integrator) on a
    sample of the headline workload: the first systems with their first
    particles, 1024 steps."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    O.build()
    sub = [(m, pel, el[:n_particles]) for m, pel, el in ensemble_elements(0)[:n_systems]]
    systems = to_cartesian(G.elements_to_cartesian, sub)

    def oracle_run(sysm):
        m, pr, pv, r, v = sysm
        ex = O.Exec(m, pr, pv, np.arange(len(m)), r, v, np.arange(len(r)), dt=180.0, tbsize=T, outer_r=300.0)
        for _ in range(blocks):
            ex.loop()
        p = ex.particles()
        o = np.argsort(p["id"])
        return {k: p[k][o] for k in ("r", "flags")}, ex.counts()["n_alive"]

    with ThreadPoolExecutor(max_workers=min(n_systems, os.cpu_count() or 1)) as pool:
        want = list(pool.map(oracle_run, systems))
    out = {}
    for name, st in (("series", G.STARTER_SERIES), ("learned", G.STARTER_LEARNED)):
        ens = make_ensemble(G, systems, T, st, path if st == G.STARTER_LEARNED else None)
        for _ in range(blocks):
            ens.step()
        worst, same = 0.0, True
        for s in range(n_systems):
            got = ens.particles(s)
            w, n_alive = want[s]
            same &= bool(np.array_equal(got["flags"], w["flags"])) and ens.counts(s)["n_alive"] == n_alive
            live = w["flags"] == 0
            d = np.linalg.norm(got["r"] - w["r"], axis=1) / np.linalg.norm(w["r"], axis=1)
            worst = max(worst, float(d[live].max()) if live.any() else 0.0)
        out[name] = {"systems": n_systems, "particles_per_system": n_particles, "steps": T * blocks,
                     "max_rel_pos_err": worst, "flags_identical": same,
                     "borderline_tests": ens.stats()["borderline"]}
        del ens
    return out


def run_headline(G, args, rank, world, path, barrier, peak_tf, local):
    """Learned + batched on the ensembles workload, the timed headline."""
    from glisser_gb300.autotune import tune_ensemble
    import torch
    systems = to_cartesian(G.elements_to_cartesian, ensemble_elements(rank, fraction=args.ensemble_fraction))
    n_total = sum(len(x[3]) for x in systems)
    if args.ensemble_shape:
        T, cta, ppt = (int(x) for x in args.ensemble_shape.split(","))
        tune = {"table": []}
    else:
        probe = to_cartesian(G.elements_to_cartesian, ensemble_elements(rank, fraction=1.0 / 16))
        tune = tune_ensemble(lambda T: make_ensemble(G, probe, T, G.STARTER_LEARNED, path),
                             time_blocks=(256, 512, 1024), blocks=2)
        T, cta, ppt = tune["best"]
    ens = make_ensemble(G, systems, T, G.STARTER_LEARNED, path, (cta, ppt))
    clocks = ClockSampler(local)
    elapsed_ms, kms, d, clk = time_ensemble(ens, args.steps, args.warmup, barrier, clocks)
    ps = d["particle_steps"]
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([elapsed_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        p = torch.tensor([float(ps)], dtype=torch.float64, device="cuda")
        dist.all_reduce(p, op=dist.ReduceOp.SUM)
        elapsed_ms, ps_all = float(t.item()), float(p.item())
    else:
        ps_all = float(ps)
    value = ps_all / (elapsed_ms * 1e-3)
    kernel_ms = sum(kms) / len(kms)
    kernel_rate = d["particle_steps"] / (sum(kms) * 1e-3)

    # end to end through the public API with host buffers: every particle's
    # r, v uploaded before and read back after each block
    r_host, v_host, _ = ens.get_state()
    barrier()
    t0 = time.perf_counter()
    ps0 = ens.stats()["particle_steps"]
    for _ in range(args.e2e_steps):
        ens.set_state(r_host, v_host)
        ens.step()
        ens.get_state(r_host, v_host)
    barrier()
    e2e_el = time.perf_counter() - t0
    e2e_ps = ens.stats()["particle_steps"] - ps0
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([e2e_el, float(e2e_ps)], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt[:1], op=dist.ReduceOp.MAX)
        dist.all_reduce(tt[1:], op=dist.ReduceOp.SUM)
        e2e_el, e2e_ps = float(tt[0].item()), float(tt[1].item())
    e2e = {"value": e2e_ps / e2e_el, "unit": UNIT, "h2d_bytes_per_step": n_total * 48,
           "d2h_bytes_per_step": n_total * (48 + 2),
           "path": "glisser_ensemble_set_state / glisser_ensemble_step / glisser_ensemble_get_state with host "
                   "[n][3] arrays (pinned staging inside the library)"}
    del ens

    # the same workload: the batched kernel with the series starter, and the
    # plain kernel one system at a time (series, and the reference's classic)
    ens = make_ensemble(G, systems, T, G.STARTER_SERIES, None, (cta, ppt))
    s_ms, s_kms, s_d, _ = time_ensemble(ens, max(2, args.steps // 2), args.warmup, barrier)
    batched_series = s_d["particle_steps"] / (s_ms * 1e-3)
    del ens
    n_plain = args.plain_systems or len(systems)
    plain_series = plain_one_at_a_time(G, systems, T, G.STARTER_SERIES, n_plain)
    plain_classic = plain_one_at_a_time(G, systems, T, G.STARTER_CLASSIC, n_plain)

    # the kernel the timed blocks ran: under the learned starter's per-block
    # dispatch the network kernel only after blocks with drifts at tau^2 >= 0.01
    variant = "learned" if d["network_blocks"] else "series"
    kernel = "batched_kernel<4,%d,%d,%s>" % (cta, ppt, variant)
    ex = executed_fp64(kernel, kernel_rate, peak_tf)
    F = alg_flops_per_particle_step(4)
    traffic = DRAM_BYTES_PER_PARTICLE_BLOCK * n_total
    roofline = {
        "bound": "fp64", "achieved": ex["achieved"] if ex else None, "peak": peak_tf, "unit": "TFLOP/s",
        "frac": ex["frac"] if ex else None, "traffic": traffic, "kernel": kernel,
        "peak_source": "measured FP64 DFMA probe on this GPU (glisser_fp64_peak_probe); MEASURED_PEAKS.json has no "
                       "FP64 figure",
        "achieved_is": "executed FP64 flops (ncu DADD + DMUL + 2 DFMA per particle-step of this build) x the "
                       "kernel's particle-step rate from CUDA events around each launch",
        "fp64_pipe_busy": ex["fp64_pipe_busy"] if ex else None, "executed": ex,
        "reference_formulation": {"flops_per_particle_step": F, "achieved": kernel_rate * F / 1e12,
                                  "frac": kernel_rate * F / 1e12 / peak_tf if peak_tf else None,
                                  "note": "the reference's algorithmic flops (five Newton passes with sin/cos "
                                          "counted as one flop each); the kernel replaces most of them, so this "
                                          "is not a lower bound and can exceed 1"},
        "traffic_is": "DRAM bytes per launch: %.0f B per particle per block (ncu) x %d particles"
                      % (DRAM_BYTES_PER_PARTICLE_BLOCK, n_total),
        "hbm_view": hbm_view(traffic, kernel_ms),
    }
    return {
        "value": value, "elapsed_ms": elapsed_ms, "kernel_ms_per_block": kernel_ms, "kernel_rate": kernel_rate,
        "particles": n_total, "time_block": T, "shape": {"threads_per_cta": cta, "particles_per_thread": ppt},
        "autotune": [{"T": a, "cta": b, "ppt": c, "rate": r} for a, b, c, r in tune["table"]],
        "gpu_launches": d["launches"], "evals_per_particle_step": d["kepler_evals"] / max(d["particle_steps"], 1),
        "network_drifts": d["learned_drifts"], "wide_drifts": d["wide_drifts"],
        "network_blocks": d["network_blocks"], "borderline_tests": d["borderline"],
        "clocks": clk, "e2e": e2e, "roofline": roofline,
        "batched_series": batched_series, "plain_series_one_at_a_time": plain_series,
        "plain_classic_one_at_a_time": plain_classic, "plain_systems_sampled": n_plain,
        "systems": systems,
    }


def hbm_view(traffic_bytes, kernel_ms):
    """The same launch against the measured HBM copy bandwidth
    (MEASURED_PEAKS.json)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        peak = json.load(open(path))["hbm_gbs"]
        src = "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, ValueError, KeyError):
        peak = 6800.0
        src = "fallback 6.8 TB/s"
    achieved = traffic_bytes / (kernel_ms * 1e-3) / 1e9
    return {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": src}


# ---------------------------------------------------------------------------
# Other legs


def timed_blocks(G, sim, blocks):
    """`blocks` blocks of a Simulation timed with CUDA events on its stream
    after one warm-up block (L2 flushed between blocks); returns rate and
    per-step counters."""
    import torch
    stream = torch.cuda.ExternalStream(sim.stream())
    sim.loop()
    s0 = sim.stats()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    kms = 0.0
    for _ in range(blocks):
        kms += sim.loop()[2]
        G.l2_flush(sim.stream(), 256 << 20)
    e1.record(stream)
    e1.synchronize()
    el = e0.elapsed_time(e1) * 1e-3
    s1 = sim.stats()
    ps = s1["particle_steps"] - s0["particle_steps"]
    return {"value": ps / el, "unit": UNIT, "kernel_ms_per_block": kms / blocks,
            "kernel_rate": ps / (kms * 1e-3), "kepler_evals_per_particle_step":
                (s1["kepler_evals"] - s0["kepler_evals"]) / max(ps, 1),
            "network_drifts": s1["learned_drifts"] - s0["learned_drifts"],
            "wide_drifts": s1["wide_drifts"] - s0["wide_drifts"],
            "network_blocks": s1["network_blocks"] - s0["network_blocks"], "particle_steps": ps,
            "borderline_tests": s1["borderline"] - s0["borderline"], "launches": s1["launches"] - s0["launches"]}


def run_plain_giants(G, args, rank, peak_tf):
    """The plain-giants workload (1e6 particles near the Neptune 3:1, Sun + 4
    giants, T = 2048): the single-system kernel with the float-float kick and
    with the FP64 kick, both against the oracle on a sample, and the
    reference's own GPU kernel on the same block."""
    from glisser_gb300 import synth
    m, pr, pv, r, v = synth.cartesian_state("plain-giants", args.particles, seed=1000 + rank)
    out = {"workload": "plain-giants: Sun + 4 giants (masses 9.55e-4, 2.86e-4, 4.37e-5, 5.15e-5 Msun), %d particles "
                       "a~U(53,57) au e~U(0,0.3) i~U(0,10deg), FP64, dt=180 d, Time-Block-Size %d; L2 flushed "
                       "between blocks" % (len(r), args.tbsize)}
    blk0 = None
    for name, kick in (("float_float_kick", G.KICK_FLOAT_FLOAT), ("fp64_kick", G.KICK_FP64)):
        sim = G.Simulation(config_text(args.tbsize, 180.0))
        sim.set_planets(m, pr, pv)
        sim.set_particles(r, v)
        sim.set_kick(kick)
        sim.init()
        if blk0 is None:
            blk0 = sim.planet_block()
        leg = timed_blocks(G, sim, args.giants_blocks)
        ex = executed_fp64("timeblock_kernel<4>", leg["kernel_rate"], peak_tf) if kick == G.KICK_FLOAT_FLOAT else None
        if ex:
            leg["executed_fp64"] = ex
        leg["vs_oracle"] = giants_vs_oracle(G, m, pr, pv, r, v, kick)
        out[name] = leg
        del sim
    out["fp64_kick_cost"] = out["float_float_kick"]["value"] / out["fp64_kick"]["value"]
    out["reference_kernel_gpu"] = reference_kernel_gpu(blk0, r, v, out["float_float_kick"]["kernel_rate"],
                                                       args.tbsize)
    return out


def giants_vs_oracle(G, m, pr, pv, r, v, kick, n=4096, steps=1024):
    """A sample of the particles over `steps` steps by the library and by the
    oracle's restatement of the reference kernel (src/wh.cu:43-177)."""
    from oracle import oracle as O
    O.build()
    sim = G.Simulation(config_text(steps, 180.0))
    sim.set_planets(m, pr, pv)
    sim.set_particles(r[:n], v[:n])
    sim.set_kick(kick)
    sim.init()
    sim.loop()
    ex = O.Exec(m, pr, pv, np.arange(len(m)), r[:n], v[:n], np.arange(n), dt=180.0, tbsize=steps)
    ex.loop()
    got, want = sim.particles(), ex.particles()
    go, wo = np.argsort(got["id"]), np.argsort(want["id"])
    live = want["flags"][wo] == 0
    d = np.linalg.norm(got["r"][go] - want["r"][wo], axis=1) / np.linalg.norm(want["r"][wo], axis=1)
    return {"particles": n, "steps": steps, "max_rel_pos_err": float(d[live].max()),
            "flags_identical": bool(np.array_equal(got["flags"][go], want["flags"][wo])),
            "borderline_tests": sim.stats()["borderline"]}


def reference_kernel_gpu(blk, r, v, ours_rate, T, launches=2):
    """The reference's own GPU time block (its src/wh.cu built unmodified for
    sm_103a by baseline/build_ref_gpu.sh; WHCudaIntegrator::
    integrate_particles_timeblock_cuda, thrust::for_each of MVSKernel) on the
    same particles and planet block, timed with CUDA events."""
    from baseline import ref_gpu
    why = ref_gpu.build()
    if why:
        return {"unavailable": why}
    g = ref_gpu.RefGpu(r, v, np.zeros_like(r), np.zeros(len(r), np.uint16), blk, 300.0, 180.0)
    g.block()                                        # warm-up launch
    ms = [g.block() for _ in range(launches)]
    out = g.download()
    rate = len(r) * T / (np.mean(ms) * 1e-3)
    return {"value": rate, "unit": UNIT, "ms_per_launch": float(np.mean(ms)), "launches": launches,
            "particles": len(r), "time_block": T, "flagged_after": int((out["flags"] != 0).sum()),
            "kernel": "the reference's MVSKernel through thrust::for_each (src/wh.cu:113-177, 344-395), built "
                      "from its sources for sm_103a with its Makefile's -O3 -maxrregcount 64",
            "timeblock_kernel_rate": ours_rate, "speedup": ours_rate / rate}


def run_scattered(G, args, rank, path, barrier):
    """The scattered disk (Sun + Neptune-mass planet; 1e6 particles a~logU(30,
    1000) au, e~U(0,0.95), i~U(0,40deg); Outer-Limit 1e5 au; Kepler tolerance
    1e-14): the classic (reference), series and learned starters, each against
    the oracle's universal-variable drift on a sample."""
    from glisser_gb300 import synth
    from oracle import oracle as O
    T = 512
    m, pr, pv, r, v = synth.cartesian_state("scattered-disk", args.learned_particles, seed=2000 + rank)
    legs = {}
    for name, st in (("classic", G.STARTER_CLASSIC), ("series", G.STARTER_SERIES), ("learned", G.STARTER_LEARNED)):
        sim = G.Simulation(config_text(T, 180.0, outer=1e5))
        sim.set_planets(m, pr, pv)
        sim.set_particles(r, v)
        sim.set_starter(st, path if st == G.STARTER_LEARNED else None)
        sim.set_kepler_tolerance(KEPLER_TOL_SCATTERED)
        sim.init()
        barrier()
        legs[name] = timed_blocks(G, sim, args.learned_blocks)
        del sim
    O.build()
    ns = 4096
    ex = O.Exec(m, pr, pv, np.arange(len(m)), r[:ns], v[:ns], np.arange(ns), dt=180.0, tbsize=T, outer_r=1e5,
                drift="uv")
    for _ in range(2):
        ex.loop()
    want = ex.particles()
    wo = np.argsort(want["id"])
    for name, st in (("classic", G.STARTER_CLASSIC), ("series", G.STARTER_SERIES), ("learned", G.STARTER_LEARNED)):
        sim = G.Simulation(config_text(T, 180.0, outer=1e5))
        sim.set_planets(m, pr, pv)
        sim.set_particles(r[:ns], v[:ns])
        sim.set_starter(st, path if st == G.STARTER_LEARNED else None)
        sim.set_kepler_tolerance(KEPLER_TOL_SCATTERED)
        sim.init()
        for _ in range(2):
            sim.loop()
        got = sim.particles()
        go = np.argsort(got["id"])
        live = want["flags"][wo] == 0
        d = np.linalg.norm(got["r"][go] - want["r"][wo], axis=1) / np.linalg.norm(want["r"][wo], axis=1)
        legs[name]["vs_oracle"] = {"particles": ns, "steps": 2 * T, "max_rel_pos_err": float(d[live].max()),
                                   "flags_identical": bool(np.array_equal(got["flags"][go], want["flags"][wo]))}
        del sim
    return {"workload": "scattered-disk: Sun + Neptune-mass planet at 30 au, %d particles a~logU(30,1000) au, "
                        "e~U(0,0.95), i~U(0,40deg), dt=180 d, Time-Block-Size %d, Outer-Limit 1e5 au, Kepler "
                        "tolerance %g" % (len(r), T, KEPLER_TOL_SCATTERED),
            "starters": legs, "learned_vs_series": legs["learned"]["value"] / legs["series"]["value"],
            "learned_vs_classic": legs["learned"]["value"] / legs["classic"]["value"]}


def run_close_eccentric(G, args, rank, barrier):
    """The regime where the learned starter runs its network on every drift:
    1e6 particles a~U(2.5,6) au, e~U(0.1,0.6) about the Sun (Neptune-mass
    planet at 30 au), dt = 180 d, so tau^2 = dt^2 mu / r^3 >= 0.0108 always.
    The network is trained on this workload's own logged plain solves; the
    series rule here is the FP32 Kepler pre-solve, the classic starter the
    reference's."""
    from glisser_gb300 import learned as L
    from glisser_gb300 import synth
    m, pr, pv, r, v = synth.cartesian_state("close-eccentric", 20000, seed=11)
    sim = G.Simulation(config_text(16, 180.0, outer=1e5))
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v)
    sim.init()
    tr = L.Trainer(20000 * 64 + 1, seed=5)
    tr.set_log_floor(L.LOG_TAU2_FLOOR)
    for _ in range(64):
        tr.log_simulation(sim)
        sim.loop()
    del sim
    tr.fit_norm()
    # this regime's targets span a wider range than the scattered disk's
    # pericentre passages: a longer run at a higher rate on larger
    # minibatches fits them to the accuracy the first Stumpff evaluation
    # accepts (loss 3e-7 against 7e-5 after the scattered disk's 8,000 steps
    # at 3e-3 on 16,384)
    losses = tr.train(args.close_train_steps, batch=args.close_batch, lr=2e-2, lr_min=1e-6, seed=3)
    path = os.path.join(tempfile.mkdtemp(), "close.bin")
    tr.save(path)
    m, pr, pv, r, v = synth.cartesian_state("close-eccentric", args.learned_particles, seed=3 + rank)
    legs = {}
    for name, st in (("classic", G.STARTER_CLASSIC), ("series", G.STARTER_SERIES), ("learned", G.STARTER_LEARNED)):
        sim = G.Simulation(config_text(512, 180.0, outer=1e5))
        sim.set_planets(m, pr, pv)
        sim.set_particles(r, v)
        sim.set_starter(st, path if st == G.STARTER_LEARNED else None)
        sim.init()
        barrier()
        legs[name] = timed_blocks(G, sim, 2)
        del sim
    # a sample against the oracle's universal-variable drift (the reference's
    # kepu spec) over two blocks, in its converged mode: at eight steps per
    # orbit the reference's acceptance (G-functions at the point whose
    # residual passed, up to 1e-13 of dt per drift) accumulates to ~1e-8 over
    # 1024 steps, so the default mode's spread is reported beside it
    from oracle import oracle as O
    O.build()
    ns = 4096
    runs = {}
    for key, conv, r_in in (("converged", True, r[:ns]), ("default", False, r[:ns]),
                            ("ulp", True, np.nextafter(r[:ns], np.inf))):
        O.set_kepu_converged(conv)
        ex = O.Exec(m, pr, pv, np.arange(len(m)), r_in, v[:ns], np.arange(ns), dt=180.0, tbsize=512,
                    outer_r=1e5, drift="uv")
        for _ in range(2):
            ex.loop()
        p = ex.particles()
        o = np.argsort(p["id"])
        runs[key] = {k: p[k][o] for k in ("r", "flags")}
        del ex
    O.set_kepu_converged(False)
    want = runs["converged"]

    def spread(x):
        return np.linalg.norm(x["r"] - want["r"], axis=1) / np.linalg.norm(want["r"], axis=1)
    for name, st in (("classic", G.STARTER_CLASSIC), ("series", G.STARTER_SERIES), ("learned", G.STARTER_LEARNED)):
        sim = G.Simulation(config_text(512, 180.0, outer=1e5))
        sim.set_planets(m, pr, pv)
        sim.set_particles(r[:ns], v[:ns])
        sim.set_starter(st, path if st == G.STARTER_LEARNED else None)
        sim.init()
        for _ in range(2):
            sim.loop()
        got = sim.particles()
        go = np.argsort(got["id"])
        live = want["flags"] == 0
        d = np.linalg.norm(got["r"][go] - want["r"], axis=1) / np.linalg.norm(want["r"], axis=1)
        legs[name]["vs_oracle"] = {"particles": ns, "steps": 1024, "max_rel_pos_err": float(d[live].max()),
                                   "q999": float(np.quantile(d[live], 0.999)),
                                   "flags_identical": bool(np.array_equal(got["flags"][go], want["flags"])),
                                   "oracle": "universal-variable drift, converged mode",
                                   "oracle_default_mode_spread": float(spread(runs["default"])[live].max()),
                                   "rounding_floor": float(spread(runs["ulp"])[live].max())}
        del sim
    out = {"workload": "close-eccentric: Sun + Neptune-mass planet at 30 au, %d particles a~U(2.5,6) au "
                       "e~U(0.1,0.6) i~U(0,20deg), dt=180 d, Time-Block-Size 512" % len(r),
           "training": {"samples": tr.samples()[0], "steps": args.close_train_steps, "batch": args.close_batch,
                        "lr": 2e-2, "loss_last": float(losses[-100:].mean())},
           "starters": legs, "learned_vs_classic": legs["learned"]["value"] / legs["classic"]["value"],
           "learned_vs_series_presolve": legs["learned"]["value"] / legs["series"]["value"]}
    if not args.no_close_ensembles:
        out["ensembles"] = run_close_ensembles(G, args, rank, path, barrier)
    return out


def run_close_ensembles(G, args, rank, path, barrier, n_systems=64, T=512):
    """Learned + batched where the network runs: 64 systems, each the Sun +
    a Neptune-mass planet (mass x U(0.9, 1.1), a x U(0.95, 1.05)), with
    close-eccentric particles (lognormal counts, median 2e4), in the batched
    kernel with the series rule (its FP32 pre-solve on every drift here) and
    with the learned starter (the close-eccentric leg's network)."""
    from glisser_gb300 import synth
    counts = synth.ensemble_counts(n_systems, seed=500 + rank)
    sub = []
    for s in range(n_systems):
        rng = np.random.default_rng(500 + rank + s)
        m, pel = synth.neptune_planets()
        m = m.copy()
        m[1] *= rng.uniform(0.9, 1.1)
        pel = pel.copy()
        pel[0, 0] *= rng.uniform(0.95, 1.05)
        sub.append((m, pel, synth.particle_elements(rng, int(counts[s]), (2.5, 6.0), (0.1, 0.6), 20.0)))
    systems = to_cartesian(G.elements_to_cartesian, sub)
    out = {"workload": "%d systems (Sun + Neptune-mass planet, mass x U(0.9,1.1), a x U(0.95,1.05)), "
                       "%d close-eccentric particles a~U(2.5,6) au e~U(0.1,0.6) i~U(0,20deg), dt=180 d, "
                       "Time-Block-Size %d, 128 threads x 1" % (n_systems, int(counts.sum()), T)}
    flags = {}
    for name, st in (("batched_series", G.STARTER_SERIES), ("batched_learned", G.STARTER_LEARNED)):
        ens = make_ensemble(G, systems, T, st, path if st == G.STARTER_LEARNED else None, (128, 1))
        el, kms, d, _ = time_ensemble(ens, 2, 2, barrier)
        out[name] = {"value": d["particle_steps"] / (el * 1e-3), "unit": UNIT,
                     "kepler_evals_per_particle_step": d["kepler_evals"] / max(d["particle_steps"], 1),
                     "network_blocks": d["network_blocks"], "network_drifts": d["learned_drifts"]}
        flags[name] = ens.get_state()[2]
        del ens
    out["learned_vs_series"] = out["batched_learned"]["value"] / out["batched_series"]["value"]
    out["flags_identical"] = bool(np.array_equal(flags["batched_series"], flags["batched_learned"]))
    return out


def run_history(G, args, rank, path, barrier):
    """Planetary history + encounter flagging: a history of the Sun +
    Neptune-mass planet (yr units) written by the library's own planet-only
    WH (dt 0.2 yr, one snapshot per 100 steps), then Neptune-crossing
    particles (a~U(20,40) au, e~U(0,0.3), i~U(0,10deg)) integrated against it
    with the history evaluated on the device each block and per-step
    3-Hill-radius encounter flags handed off through the ballot-compacted
    list; series and learned starters, and a sample against the oracle."""
    from glisser_gb300 import synth
    from oracle import oracle as O
    tmp = tempfile.mkdtemp()
    hist = os.path.join(tmp, "plhist.out")
    m, pr, pv, r, v = synth.cartesian_state("history-encounters", args.history_particles, seed=3000 + rank)
    pre = G.Simulation("Time-Step 0.2\nTime-Block-Size 100\nFinal-Time 1e9\nLimit-Particle-Count 0\n"
                       "Input-File unused\nOutput-Folder unused\n")
    pre.set_planets(m, pr, pv)
    pre.set_particles(np.zeros((0, 3)), np.zeros((0, 3)))
    pre.init()
    pre.write_plhist(hist, begin=True)
    for _ in range(2 * (1 + args.history_blocks) + 8):
        pre.loop()
        pre.write_plhist(hist)
    del pre
    cfg = ("Time-Step 0.2\nTime-Block-Size 100\nFinal-Time 1e9\nRead-Planet-History 1\nPlanet-History-File %s\n"
           "Encounter-RH-Factor 3\nCull-Radius 0.5\nOuter-Limit 300\nInput-File unused\nOutput-Folder unused\n"
           % hist)
    legs = {}
    for name, st in (("series", G.STARTER_SERIES), ("learned", G.STARTER_LEARNED)):
        sim = G.Simulation(cfg)
        sim.set_planets(m, pr, pv)
        sim.set_particles(r, v)
        sim.set_starter(st, path if st == G.STARTER_LEARNED else None)
        sim.init()
        alive0 = sim.counts()["n_alive"]
        barrier()
        leg = timed_blocks(G, sim, args.history_blocks)
        leg.update(alive_start=alive0, alive_end=sim.counts()["n_alive"])
        legs[name] = leg
        del sim
    ns = 4000
    ex = O.Exec(m, pr, pv, np.arange(len(m)), r[:ns], v[:ns], np.arange(ns), dt=0.2, tbsize=100, outer_r=300.0,
                cull_r=0.5, esf=3.0, interp_path=hist, drift="uv")
    for _ in range(10):
        ex.loop()
    want = ex.particles()
    wo = np.argsort(want["id"])
    for name, st in (("series", G.STARTER_SERIES), ("learned", G.STARTER_LEARNED)):
        sim = G.Simulation(cfg)
        sim.set_planets(m, pr, pv)
        sim.set_particles(r[:ns], v[:ns])
        sim.set_starter(st, path if st == G.STARTER_LEARNED else None)
        sim.init()
        for _ in range(10):
            sim.loop()
        got = sim.particles()
        go = np.argsort(got["id"])
        live = want["flags"][wo] == 0
        d = np.linalg.norm(got["r"][go] - want["r"][wo], axis=1) / np.linalg.norm(want["r"][wo], axis=1)
        legs[name]["vs_oracle"] = {"particles": ns, "steps": 1000, "max_rel_pos_err": float(d[live].max()),
                                   "flags_identical": bool(np.array_equal(got["flags"][go], want["flags"][wo])),
                                   "flagged": int((want["flags"] != 0).sum())}
        del sim
    return {"workload": "history-encounters: planetary history of Sun + Neptune-mass planet (a=30 au, yr units) from "
                        "the library's planet-only WH, dt=0.2 yr, one snapshot per 100 steps, evaluated on the device; "
                        "%d particles a~U(20,40) au e~U(0,0.3) i~U(0,10deg); Encounter-RH-Factor 3, Time-Block-Size "
                        "100" % len(r),
            "starters": legs, "learned_vs_series": legs["learned"]["value"] / legs["series"]["value"]}


def run_track(G, args, rank):
    """Track snapshot of a 1e6-particle state (alive particles by id, FP64
    elements, float32 records): device writer vs the host writer, wall time of
    the whole call including the file write; and the dump stream."""
    from glisser_gb300 import synth
    m, pr, pv, r, v = synth.cartesian_state("plain-giants", args.particles, seed=1000 + rank)
    sim = G.Simulation(config_text(64, 180.0))
    sim.set_planets(m, pr, pv)
    sim.set_particles(r, v)
    sim.init()
    sim.loop()
    d = "/dev/shm" if os.path.isdir("/dev/shm") else tempfile.gettempdir()
    path = os.path.join(d, "glisser_track_%d.out" % os.getpid())
    try:
        sim.write_track(path)                       # first call allocates the device buffers
        t0 = time.perf_counter()
        for _ in range(3):
            sim.write_track(path)
        dev_s = (time.perf_counter() - t0) / 3
        size = os.path.getsize(path)
        sim.set_device_output(False)
        t0 = time.perf_counter()
        sim.write_track(path)
        host_s = time.perf_counter() - t0
        sim.set_device_output(True)
    finally:
        if os.path.exists(path):
            os.remove(path)
    dpath = os.path.join(d, "glisser_dump_%d.out" % os.getpid())
    try:
        sim.set_particles(*(lambda p: (p["r"], p["v"]))(sim.particles()))    # mark the host mirror stale
        t0 = time.perf_counter()
        st = sim.particles()
        dl_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        sim.write_state(dpath, binary=True)
        wr_s = time.perf_counter() - t0
        dsize = os.path.getsize(dpath)
    finally:
        if os.path.exists(dpath):
            os.remove(dpath)
    state_bytes = len(st["r"]) * (6 * 8 + 4 + 4 + 2)
    n = sim.counts()["n_alive"]
    return {"particles": n, "bytes": size, "device_ms": dev_s * 1e3, "host_ms": host_s * 1e3,
            "device_GBps": size / dev_s / 1e9, "host_GBps": size / host_s / 1e9,
            "note": "wall time of glisser_write_track (kernels + device-to-host copy + file write to %s)" % d,
            "dump": {"download_bytes": state_bytes, "download_ms": dl_s * 1e3,
                     "download_GBps": state_bytes / dl_s / 1e9, "file_bytes": dsize, "write_ms": wr_s * 1e3,
                     "note": "glisser_get_particles after an upload (device-to-host through pinned staging and the "
                             "host mirror), then glisser_write_state binary"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="glisser", choices=["glisser", "reference"])
    ap.add_argument("--ensemble-fraction", type=float, default=1.0, help="share of each system's particles")
    ap.add_argument("--ensemble-shape", default="", help="T,cta,ppt: skip the autotuner")
    ap.add_argument("--plain-systems", type=int, default=0, help="systems run one at a time (0: all)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    # the CPU sample: ~5.4e8 particle-steps, 7-8 s on the GPU host's 16 cores
    ap.add_argument("--sample-particles", type=int, default=524288)
    ap.add_argument("--sample-steps", type=int, default=1024)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-oracle", action="store_true")
    ap.add_argument("--particles", type=int, default=1_000_000)
    ap.add_argument("--tbsize", type=int, default=2048)
    ap.add_argument("--giants-blocks", type=int, default=3)
    ap.add_argument("--no-giants", action="store_true")
    ap.add_argument("--learned-particles", type=int, default=1_000_000)
    ap.add_argument("--learned-log-blocks", type=int, default=128)
    ap.add_argument("--learned-train-steps", type=int, default=8000)
    ap.add_argument("--learned-blocks", type=int, default=3)
    ap.add_argument("--close-train-steps", type=int, default=64000)
    ap.add_argument("--close-batch", type=int, default=65536)
    ap.add_argument("--no-scattered", action="store_true")
    ap.add_argument("--no-close", action="store_true")
    ap.add_argument("--no-close-ensembles", action="store_true")
    ap.add_argument("--no-history", action="store_true")
    ap.add_argument("--history-particles", type=int, default=2_000_000)
    ap.add_argument("--history-blocks", type=int, default=20)
    ap.add_argument("--no-track", action="store_true")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import glisser_gb300 as G
    G.build()

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    peak_tf, _ = G.fp64_peak_probe()
    path, _, train_info = train_starter(G, args, rank)
    head = run_headline(G, args, rank, world, path, barrier, peak_tf, local)
    systems = head.pop("systems")

    extra = {}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        val, el, kind = reference_cpu_rate(systems, args.sample_particles, args.sample_steps, threads)
        cpu = {"value": val, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": cpu_sample_note(kind, args.sample_particles, args.sample_steps, threads) + " (%.1f s)" % el}
    if rank == 0 and not args.no_oracle:
        extra["ensembles_vs_oracle"] = ensemble_vs_oracle(G, path)
    del systems
    if not args.no_giants:
        extra["plain_giants"] = run_plain_giants(G, args, rank, peak_tf)
    if not args.no_scattered:
        extra["scattered_disk"] = run_scattered(G, args, rank, path, barrier)
    if not args.no_close:
        extra["close_eccentric"] = run_close_eccentric(G, args, rank, barrier)
    if not args.no_history:
        extra["history"] = run_history(G, args, rank, path, barrier)
    if rank == 0 and not args.no_track:
        extra["track"] = run_track(G, args, rank)

    if rank == 0:
        value = head["value"]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["elapsed_ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": ENSEMBLE_WORKLOAD + "; learned starter, batched persistent kernel, CUDA graphs",
                       "systems": 256, "particles_per_gpu": head["particles"], "time_block": head["time_block"],
                       "n_planets": 4,
                       "starter": "learned (series where it applies, network elsewhere; per-block dispatch: the "
                                  "network kernel after a block with drifts at tau^2 >= 0.01)",
                       "shape": head["shape"], "parallelism": "independent ensembles per GPU",
                       "l2": "inputs larger than L2 (%.0f MB of particle state)" % (head["particles"] * 90 / 1e6)},
            "vs_plain": value / head["plain_series_one_at_a_time"],
            "vs_plain_classic": value / head["plain_classic_one_at_a_time"],
            "vs_batched_series": value / head["batched_series"],
            "plain": {"series_one_system_per_launch": head["plain_series_one_at_a_time"],
                      "classic_one_system_per_launch": head["plain_classic_one_at_a_time"],
                      "batched_series": head["batched_series"], "systems_sampled": head["plain_systems_sampled"],
                      "note": "plain = this library's single-system time-block kernel with the series starter (its "
                              "default non-learned kernel), one system per launch as a kernel without batching "
                              "runs an ensemble; classic = the same with the reference's classic starter (the "
                              "reference's method); batched_series = the batched kernel without the network"},
            "roofline": head["roofline"],
            "kernel_ms_per_block": head["kernel_ms_per_block"],
            "kepler_evals_per_particle_step": head["evals_per_particle_step"],
            "network_drifts": head["network_drifts"], "wide_drifts": head["wide_drifts"],
            "network_blocks": head["network_blocks"], "borderline_tests": head["borderline_tests"],
            "gpu_launches": head["gpu_launches"],
            "clocks": head["clocks"],
            "e2e": head["e2e"],
            "cpu_baseline": cpu,
            "autotune": head["autotune"],
            "learned_training": train_info,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
