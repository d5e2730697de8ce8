"""Stand-in for SWIFT in the encounter hand-off tests (test infrastructure).

Called as the executor calls SWIFT: ``fake_swift.py <param> <history> <tp> <tpout>``.
It reads the integration span from the parameter file, the solar mass and the
planet count from the two-record history, the test particles from the
particle file, moves every particle on its orbit about the Sun alone (fixed
step kick-drift-kick, 8 substeps per step) and writes the output file in the
layout the hand-off reads back: the count, then per particle its position and
velocity, Swift-Status-Length integers and Swift-Status-Length reals.

What happens to a particle is a fixed function of its starting distance from
the Sun, binned at 1/8 au so that the last-digit differences between two
callers' inputs do not change it; with b = floor(8 |r0|) mod 16:

    0-8  survives, one encounter with planet 2 counted, closest approach 0.1 + b/100
    9    survives inside the inner region of planet 2 (status -2)
    10   removed, out of bounds (status -2);    11 removed, out of bounds (-3)
    12   removed, Kepler failure (-1);          13 removed, hit the Sun (1)
    14   removed, hit the second planet (2);    15 removed, hit the Sun (-4)

With FAKE_SWIFT_ARCHIVE=<dir> set, the four files of every call are copied to
<dir>/h<k>_<particle file name>, k counting the calls with that file name.
All arithmetic is IEEE add, multiply, divide and square root, so two machines
give the same output for the same input.
"""
import math
import os
import shutil
import struct
import sys

import numpy as np


def read_param(path):
    with open(path) as f:
        t0, t1, dt = (float(x) for x in f.readline().split()[:3])
    return t0, t1, dt


def read_history(path):
    with open(path, "rb") as f:
        data = f.read()
    m0 = struct.unpack_from("<d", data, 0)[0]
    npl = struct.unpack_from("<I", data, 40)[0]
    return m0, npl


def read_tp(path):
    with open(path) as f:
        tok = f.read().split()
    n = int(tok[0])
    if n == 0:
        return 0, np.zeros((0, 3)), np.zeros((0, 3)), 0
    per = (len(tok) - 1) // n
    statlen = (per - 6) // 2
    r = np.zeros((n, 3)); v = np.zeros((n, 3))
    for k in range(n):
        base = 1 + k * per
        vals = [float(x) for x in tok[base:base + 6]]
        r[k] = vals[:3]
        v[k] = vals[3:]
    return n, r, v, statlen


def accel(m0, r):
    r2 = r[:, 0] * r[:, 0] + r[:, 1] * r[:, 1] + r[:, 2] * r[:, 2]
    inv3 = 1.0 / (r2 * np.sqrt(r2))
    return -(m0 * inv3)[:, None] * r


def propagate(m0, r, v, t0, t1, dt):
    steps = max(1, int(round((t1 - t0) / dt))) * 8 if t1 > t0 else 0
    if steps == 0 or len(r) == 0:
        return r.copy(), v.copy()
    h = (t1 - t0) / steps
    r = r.copy(); v = v.copy()
    a = accel(m0, r)
    for _ in range(steps):
        v = v + a * (h / 2)
        r = r + v * h
        a = accel(m0, r)
        v = v + a * (h / 2)
    return r, v


def wrapper(dirpath):
    """Writes an executable <dirpath>/swift that runs this script with the
    current interpreter and returns its path (a test's Swift-Path)."""
    path = os.path.join(dirpath, "swift")
    with open(path, "w") as f:
        f.write('#!/bin/sh\nexec "%s" "%s" "$@"\n' % (sys.executable, os.path.abspath(__file__)))
    os.chmod(path, 0o755)
    return path


OUTCOME = {9: (0, -2), 10: (1, -2), 11: (1, -3), 12: (1, -1), 13: (1, 1), 14: (1, 2), 15: (1, -4)}


def main(argv):
    param, hist, tp, tpout = argv[1:5]
    t0, t1, dt = read_param(param)
    m0, npl = read_history(hist)
    n, r0, v0, statlen = read_tp(tp)
    r, v = propagate(m0, r0, v0, t0, t1, dt)
    lines = ["%d" % n]
    for k in range(n):
        d0 = math.sqrt(r0[k, 0] * r0[k, 0] + r0[k, 1] * r0[k, 1] + r0[k, 2] * r0[k, 2])
        b = int(math.floor(d0 * 8)) % 16
        istat = [0] * statlen
        rstat = [0.0] * statlen
        s0, s1 = OUTCOME.get(b, (0, 0))
        istat[0], istat[1], istat[2] = s0, s1, b
        rstat[0], rstat[1] = d0, t1 - t0
        if b <= 8 and statlen > 3:
            istat[3] = 1
            rstat[3] = 0.1 + b / 100.0
        if b == 14 and npl < 2:
            istat[1] = 1
        lines.append(" ".join(repr(float(x)) for x in (*r[k], *v[k])))
        lines.append(" ".join(str(x) for x in istat))
        lines.append(" ".join(repr(float(x)) for x in rstat))
    with open(tpout, "w") as f:
        f.write("\n".join(lines) + "\n")
    arch = os.environ.get("FAKE_SWIFT_ARCHIVE")
    if arch:
        os.makedirs(arch, exist_ok=True)
        name = os.path.basename(tp)
        k = sum(1 for d in os.listdir(arch) if d.endswith("_" + name))
        dst = os.path.join(arch, "h%04d_%s" % (k, name))
        os.makedirs(dst)
        for src, tag in ((param, "param"), (hist, "hist"), (tp, "tp"), (tpout, "tpout")):
            shutil.copyfile(src, os.path.join(dst, tag))
    print("fake swift: %d particles from %g to %g" % (n, t0, t1))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
