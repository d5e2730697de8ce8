"""SWIFT encounter hand-off protocol on the CPU: the files the library writes
for SWIFT and its reading of SWIFT's output, against the reference's own
SwiftEncounterIntegrator (src/swift.cpp:44-460) as recorded in
tests/golden/encounters_t50.npz (made by tests/golden/make_golden.py with
SWIFT stood in for by tests/fake_swift.py).

  - parameter and particle files: byte-identical for the same arguments;
  - history file: byte-identical layout;
  - output reading: the same state, deathflags and accumulated status arrays
    (stat.out) as the reference's end_integrate, call after call.
"""
import os

import numpy as np
import pytest

import glisser_gb300 as G

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
OUTER = 300.0        # Outer-Limit of the recorded run (the default)
STATLEN = 13         # Swift-Status-Length (the default)
PART_MIN, NUM_SWIFT = 3, 2


@pytest.fixture(scope="module")
def gold():
    G.build()
    G.lib()
    return np.load(os.path.join(GOLD, "encounters_t50.npz"))


def chunks(n):
    """begin_integrate's split of n particles over the processes."""
    nproc = max(1, min(n // PART_MIN, NUM_SWIFT))
    return [(n * i // nproc, n * (i + 1) // nproc) for i in range(nproc)]


def archive_entries(d):
    """(hand-off index, process index, archive name) of every SWIFT call."""
    calls = d["calls"]
    seen = {}
    out = []
    for k in range(len(calls)):
        for i, _ in enumerate(chunks(int(calls[k, 7]))):
            j = seen.get(i, 0)
            seen[i] = j + 1
            out.append((k, i, "h%04d_tp%d" % (j, i)))
    return out


def blob(d, name, tag):
    return d["arch_%s_%s" % (name, tag)].tobytes()


def parse_history(b):
    m0 = np.frombuffer(b, "<f8", 1, 0)[0]
    recs = []
    off = 32
    for _ in range(2):
        t = np.frombuffer(b, "<f8", 1, off)[0]
        n = int(np.frombuffer(b, "<u4", 1, off + 8)[0])
        off += 32
        ids = np.zeros(n, np.uint32); vals = np.zeros((n, 7))
        for q in range(n):
            ids[q] = np.frombuffer(b, "<u4", 1, off)[0]
            vals[q] = np.frombuffer(b, "<f4", 7, off + 4)
            off += 32
        recs.append((t, ids, vals))
    assert off == len(b)
    return m0, recs


def parse_stat(text):
    out = {}
    lines = text.strip("\n").split("\n") if text.strip() else []
    for q in range(0, len(lines), 3):
        out[int(lines[q])] = ([int(x) for x in lines[q + 1].split()], [float(x) for x in lines[q + 2].split()])
    return out


def test_archive_covers_every_handoff(gold):
    names = sorted(n for _, _, n in archive_entries(gold))
    assert names == sorted(str(x) for x in gold["archive_names"])
    calls = gold["calls"]
    assert (calls[:, 0] == 0).any() and (calls[:, 0] == 1).any()   # mid-interval and end-of-interval hand-offs
    assert any(len(chunks(int(n))) == 2 for n in calls[:, 7])        # two processes at least once


def test_param_and_particle_files_match(gold, tmp_path):
    calls = gold["calls"]
    for k, i, name in archive_entries(gold):
        _, _, rel_t, dt, prev_len, cur_len, _, n = calls[k]
        p = str(tmp_path / "param")
        G.swift_write_param(p, rel_t, int(prev_len), int(cur_len), dt, OUTER)
        assert open(p, "rb").read() == blob(gold, name, "param"), name
        b, e = chunks(int(n))[i]
        tp = str(tmp_path / "tp")
        G.swift_write_tp(tp, gold["call%d_r_in" % k][b:e], gold["call%d_v_in" % k][b:e], STATLEN)
        assert open(tp, "rb").read() == blob(gold, name, "tp"), name


def test_history_file_layout(gold, tmp_path):
    for _, _, name in archive_entries(gold)[:6]:
        ref = blob(gold, name, "hist")
        m0, ((t0, ids0, v0), (t1, ids1, v1)) = parse_history(ref)
        assert t0 == 0.0 and t1 > 0 and np.array_equal(ids0, ids1)
        h = str(tmp_path / "hist")
        G.swift_write_history(h, m0, t1, ids0 - 1, v0[:, 0], v0[:, 1:4], v0[:, 4:7], v1[:, 1:4], v1[:, 4:7])
        assert open(h, "rb").read() == ref, name


def test_output_reading_matches_end_integrate(gold, tmp_path):
    st = G.SwiftStats(STATLEN)
    calls = gold["calls"]
    entries = archive_entries(gold)
    for k in range(len(calls)):
        n = int(calls[k, 7])
        ids = gold["call%d_ids" % k]
        r = np.zeros((n, 3)); v = np.zeros((n, 3)); fl = np.zeros(n, np.uint16)
        for kk, i, name in entries:
            if kk != k:
                continue
            b, e = chunks(n)[i]
            _, ((_, pid, _), _) = parse_history(blob(gold, name, "hist"))
            path = str(tmp_path / "tpout")
            with open(path, "wb") as f:
                f.write(blob(gold, name, "tpout"))
            r[b:e], v[b:e], fl[b:e] = st.read_tpout(path, ids[b:e], pid - 1)
        np.testing.assert_array_equal(r, gold["call%d_r_out" % k])
        np.testing.assert_array_equal(v, gold["call%d_v_out" % k])
        np.testing.assert_array_equal(fl, gold["call%d_flags" % k])
    path = str(tmp_path / "stat.out")
    st.write(path)
    ours = parse_stat(open(path).read())
    ref = parse_stat(str(gold["stat_out"]))
    assert ours == ref
    # same line format per particle (the reference's order is its hash map's)
    ref_lines = str(gold["stat_out"]).strip("\n").split("\n")
    our_lines = open(path).read().strip("\n").split("\n")
    ref_blocks = {ref_lines[q]: ref_lines[q:q + 3] for q in range(0, len(ref_lines), 3)}
    for q in range(0, len(our_lines), 3):
        assert our_lines[q:q + 3] == ref_blocks[our_lines[q]]
    ist, rst = st.get(int(ids[0]))
    assert ist.tolist() == ref[int(ids[0])][0]
    assert st.get(0xFFFFFFF0) is None


def test_output_reading_errors(tmp_path):
    G.build()
    st = G.SwiftStats(STATLEN)
    p = str(tmp_path / "tpout")
    row = "1.0 2.0 3.0 0.1 0.2 0.3\n" + " ".join(["0"] * STATLEN) + "\n" + " ".join(["0.0"] * STATLEN) + "\n"
    with open(p, "w") as f:
        f.write("2\n" + row)
    with pytest.raises(G.GlisserError):           # count mismatch
        st.read_tpout(p, np.array([1], np.uint32), np.array([1, 2], np.uint32))
    with open(p, "w") as f:
        f.write("1\n1.0 2.0 oops\n")
    with pytest.raises(G.GlisserError):           # malformed
        st.read_tpout(p, np.array([1], np.uint32), np.array([1, 2], np.uint32))
    bad = "1\n1.0 2.0 3.0 0.1 0.2 0.3\n1 7 " + " ".join(["0"] * (STATLEN - 2)) + "\n" + \
        " ".join(["0.0"] * STATLEN) + "\n"
    with open(p, "w") as f:
        f.write(bad)
    with pytest.raises(G.GlisserError):           # planet 7 is not in a two-planet list
        st.read_tpout(p, np.array([1], np.uint32), np.array([1, 2], np.uint32))
    with open(p, "w") as f:
        f.write("1\n" + row)
    r, v, fl = st.read_tpout(p, np.array([1], np.uint32), np.array([1, 2], np.uint32))
    assert fl[0] == 0 and r[0].tolist() == [1.0, 2.0, 3.0]
