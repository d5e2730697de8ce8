"""Generates the golden fixtures in tests/golden/ by running the UNMODIFIED
reference sources (compiled by oracle/build_ref.sh into oracle/_ref/).

Run where the reference checkout is available:
    GLISSER_REF_DIR=<reference checkout> python tests/golden/make_golden.py
Only this script reads the reference; the fixtures it writes are what the
tests (here and on the GPU host) compare against.
"""
import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from glisser_gb300 import synth  # noqa: E402
from glisser_gb300.metrics import jacobi_constant  # noqa: E402

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libglisser_ref.so")
REFERENCE = os.environ.get("GLISSER_REF_DIR")
if not REFERENCE:
    sys.exit("make_golden.py: set GLISSER_REF_DIR to the reference checkout")
D = C.POINTER(C.c_double)
U32 = C.POINTER(C.c_uint32)
U16 = C.POINTER(C.c_uint16)


def ref():
    if not os.path.exists(REF_LIB):
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    L = C.CDLL(REF_LIB)
    L.ref_kepu.argtypes = [C.c_double] * 5 + [D] * 4
    L.ref_kepu.restype = C.c_int
    L.ref_from_elements_M.argtypes = [C.c_double] * 7 + [D, D]
    L.ref_to_elements.argtypes = [C.c_double, D, D, C.POINTER(C.c_int), D]
    L.ref_mean_anomaly.argtypes = [C.c_double, C.c_double]
    L.ref_mean_anomaly.restype = C.c_double
    L.ref_exec_create.argtypes = [C.c_char_p]
    L.ref_exec_create.restype = C.c_void_p
    L.ref_exec_destroy.argtypes = [C.c_void_p]
    L.ref_exec_init.argtypes = [C.c_void_p]
    L.ref_exec_loop.argtypes = [C.c_void_p]
    L.ref_exec_error.argtypes = [C.c_void_p]
    L.ref_exec_error.restype = C.c_char_p
    L.ref_exec_counts.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), D,
                                  C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    L.ref_exec_particles.argtypes = [C.c_void_p, D, D, D, U32, U16, U32, D]
    L.ref_exec_planet_block.argtypes = [C.c_void_p, D, D, D, U32, D]
    L.ref_exec_planets.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), D, D, D, U32]
    L.ref_exec_save_state.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    L.ref_exec_write_track.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_int]
    L.ref_exec_write_plhist.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    L.ref_exec_encounter_log.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
    L.ref_exec_encounter_log.restype = C.c_size_t
    L.ref_write_config.argtypes = [C.c_char_p, C.c_char_p]
    L.ref_check_config.argtypes = [C.c_char_p, C.c_char_p, C.c_size_t]
    L.ref_mvs_block.argtypes = [C.c_size_t, D, D, D, U16, U32, C.c_uint32, C.c_uint32, D, D, D, U32, D,
                                C.c_double, C.c_double, C.c_double]
    return L


def p(a, t):
    return a.ctypes.data_as(t)


def cartesian(L, mu, el):
    r = np.zeros((len(el), 3))
    v = np.zeros((len(el), 3))
    for k, e in enumerate(el):
        L.ref_from_elements_M(mu, *map(float, e), p(r[k], D), p(v[k], D))
    return r, v


def write_state(path, pl_m, pl_r, pl_v, r, v, ids=None, flags=None):
    """ASCII hybrid state (the layout load_data_hybrid reads, src/data.cpp:427-483)."""
    n = len(r)
    ids = np.arange(n) if ids is None else ids
    flags = np.zeros(n, int) if flags is None else flags
    with open(path, "w") as f:
        f.write("%d\n" % len(pl_m))
        for i in range(len(pl_m)):
            f.write("%.17g\n%.17g %.17g %.17g\n%.17g %.17g %.17g\n%d\n" % (pl_m[i], *pl_r[i], *pl_v[i], i))
        f.write("%d\n" % n)
        for k in range(n):
            f.write("%.17g %.17g %.17g\n%.17g %.17g %.17g\n%d %d 0\n" % (*r[k], *v[k], ids[k], flags[k]))


class RefRun:
    def __init__(self, L, config_text):
        self.L = L
        self.h = L.ref_exec_create(config_text.encode())
        if not self.h:
            raise RuntimeError("reference could not load the run")
        if L.ref_exec_init(self.h):
            raise RuntimeError(L.ref_exec_error(self.h).decode())

    def loop(self):
        if self.L.ref_exec_loop(self.h):
            raise RuntimeError(self.L.ref_exec_error(self.h).decode())

    def counts(self):
        n, na = C.c_size_t(), C.c_size_t()
        t = C.c_double()
        npl, ln = C.c_uint32(), C.c_uint32()
        self.L.ref_exec_counts(self.h, C.byref(n), C.byref(na), C.byref(t), C.byref(npl), C.byref(ln))
        return n.value, na.value, t.value, npl.value, ln.value

    def particles(self):
        n = self.counts()[0]
        r = np.zeros((n, 3)); v = np.zeros((n, 3)); a = np.zeros((n, 3))
        ids = np.zeros(n, np.uint32); fl = np.zeros(n, np.uint16); dti = np.zeros(n, np.uint32); dt = np.zeros(n)
        self.L.ref_exec_particles(self.h, p(r, D), p(v, D), p(a, D), p(ids, U32), p(fl, U16), p(dti, U32), p(dt, D))
        return dict(r=r, v=v, a=a, id=ids, flags=fl, dti=dti, deathtime=dt)

    def planet_block(self):
        _, _, _, npl, ln = self.counts()
        r_log = np.zeros((ln, npl - 1, 3)); h0 = np.zeros((ln, 3))
        m = np.zeros(npl); ids = np.zeros(npl, np.uint32); rh = np.zeros(npl)
        self.L.ref_exec_planet_block(self.h, p(r_log, D), p(h0, D), p(m, D), p(ids, U32), p(rh, D))
        return dict(r_log=r_log, h0_log=h0, m=m, id=ids, rh=rh)

    def planets(self):
        n = C.c_size_t()
        m = np.zeros(64); r = np.zeros((64, 3)); v = np.zeros((64, 3)); ids = np.zeros(64, np.uint32)
        self.L.ref_exec_planets(self.h, C.byref(n), p(m, D), p(r, D), p(v, D), p(ids, U32))
        k = n.value
        return m[:k], r[:k], v[:k], ids[:k]

    def encounter_log(self):
        sz = self.L.ref_exec_encounter_log(self.h, None, 0)
        buf = C.create_string_buffer(sz + 1)
        self.L.ref_exec_encounter_log(self.h, buf, sz + 1)
        return buf.value.decode()


def run_case(L, tmp, name, config_lines, pl_m, pl_r, pl_v, r, v, nblocks, out):
    state = os.path.join(tmp, name + ".state.in")
    write_state(state, pl_m, pl_r, pl_v, r, v)
    cfg = "\n".join(config_lines + ["Input-File " + state, "Output-Folder " + tmp]) + "\n"
    run = RefRun(L, cfg)
    rec = dict(pl_m=pl_m, pl_r=pl_r, pl_v=pl_v, r0=r, v0=v)
    p0 = run.particles()
    rec["a0"] = p0["a"]
    rec["flags0"] = p0["flags"]
    for b in range(nblocks):
        blk = run.planet_block()
        for k in ("r_log", "h0_log", "m", "id", "rh"):
            rec["blk%d_%s" % (b, k)] = blk[k]
        run.loop()
        st = run.particles()
        n, na, t, _, _ = run.counts()
        for k in ("r", "v", "a", "id", "flags", "dti", "deathtime"):
            rec["out%d_%s" % (b, k)] = st[k]
        rec["out%d_n_alive" % b] = np.array(na)
        rec["out%d_t" % b] = np.array(t)
    pm, pr, pv, pid = run.planets()
    rec.update(final_pl_m=pm, final_pl_r=pr, final_pl_v=pv, final_pl_id=pid)
    rec["encounter_log"] = np.array(run.encounter_log())
    rec["config"] = np.array("\n".join(config_lines))
    rec["nblocks"] = np.array(nblocks)
    np.savez_compressed(os.path.join(HERE, out), **rec)
    print("wrote", out, "alive after each block:", [int(rec["out%d_n_alive" % b]) for b in range(nblocks)])
    return run


def gen_threebody(L):
    """The reference's own restricted three-body example
    (example/threebody-particles/state.in.full: 1000 particles; Sun, a
    massless body at 5.2 au and a 2.04e-3 primary at 30.4 au, yr units) run by
    the reference for 50 blocks of 100 steps of 0.2 yr (1000 yr) with
    Encounter-RH-Factor 3.5, as in example/threebody-particles/config.in."""
    state = os.path.join(REFERENCE, "example", "threebody-particles", "state.in.full")
    lines = ["Time-Step 0.2", "Time-Block-Size 100", "Final-Time 1000", "Encounter-RH-Factor 3.5",
             "Cull-Radius 0.5"]
    cfg = "\n".join(lines + ["Input-File " + state, "Output-Folder /tmp"]) + "\n"
    run = RefRun(L, cfg)
    pm, pr, pv, pid = run.planets()
    p0 = run.particles()
    rec = dict(pl_m=pm, pl_r=pr, pl_v=pv, pl_id=pid, r0=p0["r"], v0=p0["v"], id0=p0["id"], flags0=p0["flags"],
               config=np.array("\n".join(lines)))
    o = np.argsort(p0["id"])
    c0 = jacobi_constant(pm, pr, pv, p0["r"][o], p0["v"][o])
    maxerr = np.zeros(len(o))
    for b in range(50):
        run.loop()
        st = run.particles()
        m_, r_, v_, _ = run.planets()
        o = np.argsort(st["id"])
        c = jacobi_constant(m_, r_, v_, st["r"][o], st["v"][o])
        live = st["flags"][o] == 0
        maxerr = np.where(live, np.maximum(maxerr, np.abs(c - c0) / np.abs(c0)), maxerr)
        if b in (4, 49):
            for k in ("r", "v", "id", "flags", "dti"):
                rec["out%d_%s" % (b, k)] = st[k]
            rec["out%d_n_alive" % b] = np.array(run.counts()[1])
    rec["cj0"] = c0
    rec["cj_maxerr"] = maxerr
    np.savez_compressed(os.path.join(HERE, "threebody_t100.npz"), **rec)
    live = rec["out49_flags"] == 0
    print("wrote threebody_t100.npz: alive after 5 / 50 blocks", int(rec["out4_n_alive"]), int(rec["out49_n_alive"]),
          "max C_J error (alive)", maxerr[np.sort(rec["out49_id"][live])].max())


def main():
    L = ref()
    tmp = tempfile.mkdtemp(prefix="glisser_golden_")

    # --- plain-neptune shape: Sun + Neptune-mass planet, 200 particles, 8 blocks of 128
    w = synth.workload("plain-neptune", n=200, seed=0)
    m = w["pl_m"]
    prr, pvv = cartesian(L, m[0] + m[1], w["pl_el"])
    pl_r = np.vstack([np.zeros(3), prr]); pl_v = np.vstack([np.zeros(3), pvv])
    r, v = cartesian(L, m[0], w["el"])
    run_case(L, tmp, "neptune", ["Time-Step 180", "Time-Block-Size 128", "Final-Time 1e9"],
             m, pl_r, pl_v, r, v, 8, "neptune_t128.npz")

    # --- plain-giants shape: Sun + four giants, 128 particles near the 3:1, 4 blocks of 256
    w = synth.workload("plain-giants", n=128, seed=0)
    m = w["pl_m"]
    pl_r = [np.zeros(3)]; pl_v = [np.zeros(3)]
    for k in range(4):
        a, b = cartesian(L, m[0] + m[k + 1], w["pl_el"][k:k + 1])
        pl_r.append(a[0]); pl_v.append(b[0])
    pl_r = np.array(pl_r); pl_v = np.array(pl_v)
    r, v = cartesian(L, m[0], w["el"])
    run_case(L, tmp, "giants", ["Time-Step 180", "Time-Block-Size 256", "Final-Time 1e9"],
             m, pl_r, pl_v, r, v, 4, "giants_t256.npz")

    # --- flag-heavy case: eccentric Neptune crossers, wide cull radius, near outer limit
    rng = np.random.default_rng(7)
    m, pel = synth.neptune_planets()
    prr, pvv = cartesian(L, m[0] + m[1], pel)
    pl_r = np.vstack([np.zeros(3), prr]); pl_v = np.vstack([np.zeros(3), pvv])
    el = synth.particle_elements(rng, 256, (20, 45), (0.2, 0.9), 10.0)
    r, v = cartesian(L, m[0], el)
    run_case(L, tmp, "flags", ["Time-Step 180", "Time-Block-Size 64", "Final-Time 1e9",
                               "Cull-Radius 2.5", "Outer-Limit 60"],
             m, pl_r, pl_v, r, v, 6, "flags_t64.npz")

    # --- Hill-sphere encounters by planet id (Encounter-RH-Factor > 0), 4 giants
    rng = np.random.default_rng(11)
    w = synth.workload("plain-giants", n=4, seed=3)
    m = w["pl_m"]
    pl_r = [np.zeros(3)]; pl_v = [np.zeros(3)]
    for k in range(4):
        a, b = cartesian(L, m[0] + m[k + 1], w["pl_el"][k:k + 1])
        pl_r.append(a[0]); pl_v.append(b[0])
    pl_r = np.array(pl_r); pl_v = np.array(pl_v)
    el = synth.particle_elements(rng, 256, (6, 32), (0.0, 0.5), 5.0)
    r, v = cartesian(L, m[0], el)
    run_case(L, tmp, "hill", ["Time-Step 60", "Time-Block-Size 64", "Final-Time 1e9",
                              "Encounter-RH-Factor 3", "Cull-Radius 1"],
             m, pl_r, pl_v, r, v, 6, "hill_t64.npz")

    # --- planetary history: planets-only run in yr units writing plhist every 25 blocks of 4 steps
    m, pel = synth.neptune_planets(synth.GM_SUN_AU_YR, a=30.4)
    m = np.array([m[0], 1e-24, m[1]])
    pel = np.array([[5.2, 0, 0, 0, 0, 0], [30.4, 0, 0, 0, 0, 0]])
    pl_r = [np.zeros(3)]; pl_v = [np.zeros(3)]
    for k in range(2):
        a, b = cartesian(L, m[0] + m[k + 1], pel[k:k + 1])
        pl_r.append(a[0]); pl_v.append(b[0])
    pl_r = np.array(pl_r); pl_v = np.array(pl_v)
    state = os.path.join(tmp, "hist.state.in")
    write_state(state, m, pl_r, pl_v, np.zeros((0, 3)), np.zeros((0, 3)))
    plh = os.path.join(HERE, "plhist_yr.bin")
    run = RefRun(L, "Time-Step 0.2\nTime-Block-Size 5\nFinal-Time 1e9\nLimit-Particle-Count 0\n"
                    "Input-File %s\nOutput-Folder %s\n" % (state, tmp))
    L.ref_exec_write_plhist(run.h, plh.encode(), 1)
    for b in range(20 * 40):
        run.loop()
        if (b + 1) % 20 == 0:
            L.ref_exec_write_plhist(run.h, plh.encode(), 0)
    print("wrote plhist_yr.bin", os.path.getsize(plh), "bytes")

    rng = np.random.default_rng(5)
    el = synth.particle_elements(rng, 256, (20, 40), (0.0, 0.3), 10.0)
    r, v = cartesian(L, m[0], el)
    run_case(L, tmp, "interp", ["Time-Step 0.2", "Time-Block-Size 50", "Final-Time 1e9",
                                "Read-Planet-History 1", "Planet-History-File " + plh,
                                "Encounter-RH-Factor 3", "Cull-Radius 0.5"],
             m, pl_r, pl_v, r, v, 10, "interp_t50.npz")

    # --- universal-variable solver on a grid (elliptic and hyperbolic)
    rng = np.random.default_rng(3)
    nk = 4000
    mu = np.where(rng.random(nk) < 0.5, synth.GM_SUN_AU_DAY, synth.GM_SUN_AU_YR)
    r0 = np.exp(rng.uniform(np.log(0.5), np.log(2000), nk))
    vcirc = np.sqrt(mu / r0)
    vv = vcirc * rng.uniform(0.05, 1.6, nk)
    alpha = 2 * mu / r0 - vv ** 2
    u = r0 * vv * rng.uniform(-1, 1, nk)
    period = 2 * np.pi * np.sqrt(r0 ** 3 / mu)
    dt = period * np.exp(rng.uniform(np.log(1e-5), np.log(0.3), nk))
    out = np.zeros((nk, 5))
    for k in range(nk):
        fp, c1, c2, c3 = (C.c_double() for _ in range(4))
        fail = L.ref_kepu(dt[k], r0[k], mu[k], alpha[k], u[k], C.byref(fp), C.byref(c1), C.byref(c2), C.byref(c3))
        out[k] = (fail, fp.value, c1.value, c2.value, c3.value)
    np.savez_compressed(os.path.join(HERE, "kepu_grid.npz"), dt=dt, r0=r0, mu=mu, alpha=alpha, u=u, out=out)
    print("wrote kepu_grid.npz, failures:", int(out[:, 0].sum()))

    # --- element conversions
    rng = np.random.default_rng(4)
    ne = 2000
    el = np.stack([rng.uniform(1, 100, ne), rng.uniform(0, 0.99, ne), rng.uniform(0, np.pi, ne),
                   rng.uniform(0, 2 * np.pi, ne), rng.uniform(0, 2 * np.pi, ne), rng.uniform(-10, 10, ne)], 1)
    mu = synth.GM_SUN_AU_DAY
    rr, vv = cartesian(L, mu, el)
    back = np.zeros((ne, 6)); esign = np.zeros(ne, np.int32)
    for k in range(ne):
        es = C.c_int()
        L.ref_to_elements(mu, p(rr[k], D), p(vv[k], D), C.byref(es), p(back[k], D))
        esign[k] = es.value
    manom = np.array([L.ref_mean_anomaly(el[k, 1], back[k, 5]) for k in range(ne)])
    np.savez_compressed(os.path.join(HERE, "elements.npz"), mu=mu, el=el, r=rr, v=vv, back=back, esign=esign,
                        manom=manom)
    print("wrote elements.npz")

    # --- file formats written by the reference writers
    w = synth.workload("plain-neptune", n=40, seed=2)
    m = w["pl_m"]
    prr, pvv = cartesian(L, m[0] + m[1], w["pl_el"])
    pl_r = np.vstack([np.zeros(3), prr]); pl_v = np.vstack([np.zeros(3), pvv])
    r, v = cartesian(L, m[0], w["el"])
    r[3] = [500.0, 0, 0]   # one particle starts beyond the outer limit: flagged 0x02 at init
    run = run_case(L, tmp, "fmt", ["Time-Step 180", "Time-Block-Size 16", "Final-Time 1e9", "Outer-Limit 300"],
                   m, pl_r, pl_v, r, v, 2, "formats_run.npz")
    L.ref_exec_save_state(run.h, os.path.join(HERE, "state_ascii.out").encode(), 0)
    L.ref_exec_save_state(run.h, os.path.join(HERE, "state_binary.out").encode(), 1)
    L.ref_exec_write_track(run.h, os.path.join(HERE, "track_bary.out").encode(), 0, 1)
    L.ref_exec_write_track(run.h, os.path.join(HERE, "track_helio.out").encode(), 0, 0)
    L.ref_exec_write_plhist(run.h, os.path.join(HERE, "plhist_fmt.out").encode(), 1)
    cfg_text = ("Initial-Time 3\nTime-Step 0.5\nFinal-Time 99\nTime-Block-Size 64\nEncounter-RH-Factor 3.5\n"
                "Cull-Radius 0.25\nOuter-Limit 1000\nLog-Interval 7\nTrack-Interval 3\nDump-Interval 11\n"
                "Input-File in.txt\nOutput-File out.txt\nOutput-Folder some/where\nSwift-Process-Count 3\n"
                "Write-Barycentric-Track 0\nBig-G 2\n")
    with open(os.path.join(HERE, "config_in.txt"), "w") as f:
        f.write(cfg_text)
    L.ref_write_config(cfg_text.encode(), os.path.join(HERE, "config_written.txt").encode())

    bad = [
        "Time-Step\n",
        "Bogus-Key 3\nInput-File x\n",
        "Time-Step abc\nInput-File x\n",
        "Output-File \nInput-File x\n",
        "Resync-Interval 2\nResolve-Encounters 1\nInput-File x\n",
        "Time-Step 1\n",
        "Read-Split-Input 1\nInput-File x\n",
        "Resolve-Encounters 1\nInput-File x\n",
    ]
    msgs = []
    for b in bad:
        buf = C.create_string_buffer(512)
        rc = L.ref_check_config(b.encode(), buf, 512)
        msgs.append("%d\t%s" % (rc, buf.value.decode()))
    with open(os.path.join(HERE, "config_errors.txt"), "w") as f:
        for b, mm in zip(bad, msgs):
            f.write(repr(b) + "\t" + mm + "\n")
    print("wrote format fixtures")


ENCOUNTER_CONFIG = ["Time-Step 0.2", "Time-Block-Size 50", "Final-Time 1e9", "Read-Planet-History 1",
                    "Encounter-RH-Factor 3", "Cull-Radius 0.5", "Resolve-Encounters 1", "Swift-Process-Count 2",
                    "Swift-Process-Min-Particle-Count 3"]


def encounter_config(plh, swift, out):
    return "\n".join(ENCOUNTER_CONFIG + ["Planet-History-File " + plh, "Swift-Path " + swift,
                                         "Output-Folder " + out])


def encounter_particles(L, n=600, seed=21):
    """Particles on near-circular orbits across Neptune's in plhist_yr.bin."""
    m, _ = synth.neptune_planets(synth.GM_SUN_AU_YR, a=30.4)
    rng = np.random.default_rng(seed)
    el = synth.particle_elements(rng, n, (28, 33), (0.0, 0.1), 5.0)
    return cartesian(L, m[0], el)


def gen_encounters(L, nblocks=24):
    """Resolve-Encounters: the reference's own hand-off
    (SwiftEncounterIntegrator, src/swift.cpp) under the restated executor loop,
    with SWIFT stood in for by tests/fake_swift.py.  Records every block's
    counts, the final state, encounter.out, stat.out, each hand-off's
    arguments and data, and the files of every SWIFT call."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import fake_swift
    wdir = tempfile.mkdtemp(prefix="glisser_enc_")
    swift = fake_swift.wrapper(wdir)
    arch = os.path.join(wdir, "archive")
    os.environ["FAKE_SWIFT_ARCHIVE"] = arch
    out = os.path.join(wdir, "out")
    os.makedirs(out)
    plh = os.path.join(HERE, "plhist_yr.bin")
    m, _ = synth.neptune_planets(synth.GM_SUN_AU_YR, a=30.4)
    m = np.array([m[0], 1e-24, m[1]])
    pl_r = np.zeros((3, 3)); pl_v = np.zeros((3, 3))
    pl_r[1, 0] = 5.2; pl_r[2, 0] = 30.4   # replaced by the history's first record
    r, v = encounter_particles(L)
    state = os.path.join(wdir, "enc.state.in")
    cfg = encounter_config(plh, swift, out)
    # particles that start inside an encounter radius would be flagged at init
    # (and the reference leaves their accelerations in load order): leave them out
    write_state(state, m, pl_r, pl_v, r, v)
    run = RefRun(L, cfg + "\nInput-File " + state + "\n")
    f0 = run.particles()["flags"]
    keep = np.sort(run.particles()["id"][f0 == 0])
    r, v = r[keep], v[keep]
    ids = keep.astype(np.uint32)
    write_state(state, m, pl_r, pl_v, r, v, ids=ids)
    run = RefRun(L, cfg + "\nInput-File " + state + "\n")
    L.ref_exec_counts2.argtypes = [C.c_void_p] + [C.POINTER(C.c_size_t)] * 3
    L.ref_exec_swift_calls.argtypes = [C.c_void_p]
    L.ref_exec_swift_calls.restype = C.c_size_t
    L.ref_exec_swift_call.argtypes = [C.c_void_p, C.c_size_t, C.POINTER(C.c_int), D, C.POINTER(C.c_size_t)]
    L.ref_exec_swift_call_data.argtypes = [C.c_void_p, C.c_size_t, U32, D, D, D, D, U16]
    L.ref_exec_write_stat.argtypes = [C.c_void_p, C.c_char_p]
    rec = dict(pl_m=m, pl_r=pl_r, pl_v=pl_v, r0=r, v0=v, id0=ids, nblocks=np.array(nblocks),
               config=np.array("\n".join(ENCOUNTER_CONFIG)))
    counts = []
    for b in range(nblocks):
        run.loop()
        da, ha, ne = C.c_size_t(), C.c_size_t(), C.c_size_t()
        L.ref_exec_counts2(run.h, C.byref(da), C.byref(ha), C.byref(ne))
        counts.append((run.counts()[2], da.value, ha.value, ne.value))
    rec["counts"] = np.array(counts)
    st = run.particles()
    for k in ("r", "v", "id", "flags", "deathtime"):
        rec["out_" + k] = st[k]
    rec["encounter_log"] = np.array(run.encounter_log())
    stat = os.path.join(wdir, "stat.out")
    L.ref_exec_write_stat(run.h, stat.encode())
    rec["stat_out"] = np.array(open(stat).read())
    ncall = L.ref_exec_swift_calls(run.h)
    meta = np.zeros((ncall, 8))
    for k in range(ncall):
        old = C.c_int(); t3 = np.zeros(3); sz = (C.c_size_t * 4)()
        L.ref_exec_swift_call(run.h, k, C.byref(old), p(t3, D), sz)
        meta[k] = (old.value, *t3, *list(sz))
        n = sz[3]
        ids_k = np.zeros(n, np.uint32); fl = np.zeros(n, np.uint16)
        arrs = [np.zeros((n, 3)) for _ in range(4)]
        L.ref_exec_swift_call_data(run.h, k, p(ids_k, U32), *[p(a, D) for a in arrs], p(fl, U16))
        rec["call%d_ids" % k] = ids_k
        for nm, a in zip(("r_in", "v_in", "r_out", "v_out"), arrs):
            rec["call%d_%s" % (k, nm)] = a
        rec["call%d_flags" % k] = fl
    rec["calls"] = meta   # old, t, rel_t, dt, prev_len, cur_len, begin, n
    names = sorted(os.listdir(arch))
    rec["archive_names"] = np.array(names)
    for nm in names:
        for tag in ("param", "hist", "tp", "tpout"):
            with open(os.path.join(arch, nm, tag), "rb") as f:
                rec["arch_%s_%s" % (nm, tag)] = np.frombuffer(f.read(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "encounters_t50.npz"), **rec)
    del os.environ["FAKE_SWIFT_ARCHIVE"]
    print("wrote encounters_t50.npz: %d particles, %d hand-offs, %d SWIFT calls; counts per block:"
          % (len(ids), ncall, len(names)), [tuple(int(x) for x in c[1:]) for c in counts])


if __name__ == "__main__":
    if sys.argv[1:] == ["threebody"]:
        gen_threebody(ref())
    elif sys.argv[1:] == ["encounters"]:
        gen_encounters(ref())
    else:
        main()
        gen_threebody(ref())
        gen_encounters(ref())
