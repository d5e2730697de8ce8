"""Multi-process runs: one process per GPU, each integrating a contiguous id
range of the particles against the same planets.

Particles are independent given the planet log, so the shards never
exchange data while they integrate: every rank builds the (tiny) planet log
itself.  At an output interval the ranks exchange only host metadata -- the
alive/encounter counts and the compacted flagged-particle lists of the block,
gathered on rank 0 -- and rank 0 merges the per-rank track snapshots by id
into the single-process track layout (save_binary_track,
src/data.cpp:718-815: time, planet count, planet records, particle count,
particle records sorted by id).

The exchange uses a torch.distributed process group on the host (gloo);
no collective touches device memory.
"""
import struct

import numpy as np

TRACK_RECORD = np.dtype([("id", "<u4"), ("el", "<f4", (6,))])    # 28 bytes, packed


def shard_bounds(n, rank, world):
    """[lo, hi) of rank's contiguous share of n particles."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside world %d" % (rank, world))
    return n * rank // world, n * (rank + 1) // world


def shard(rank, world, *arrays):
    """Rank's contiguous slice of each array (all of the same length)."""
    n = len(arrays[0])
    lo, hi = shard_bounds(n, rank, world)
    return tuple(a[lo:hi] for a in arrays)


def gather_block(counts, flagged, group=None, dst=0):
    """Gathers one block's metadata on rank `dst`: counts (dict of n, n_alive,
    n_encounter) are summed and the flagged lists (dict of id, flags,
    deathtime_index arrays) are concatenated and ordered by id.  Returns the
    merged (counts, flagged) on dst and None elsewhere."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    payload = ({k: int(v) for k, v in counts.items()},
               {k: np.asarray(v) for k, v in flagged.items()})
    out = [None] * world if rank == dst else None
    dist.gather_object(payload, out, dst=dst, group=group)
    if rank != dst:
        return None
    total = {}
    for c, _ in out:
        for k, v in c.items():
            total[k] = total.get(k, 0) + v
    keys = out[0][1].keys()
    merged = {k: np.concatenate([f[k] for _, f in out]) for k in keys}
    if "id" in merged and len(merged["id"]):
        o = np.argsort(merged["id"], kind="stable")
        merged = {k: v[o] for k, v in merged.items()}
    return total, merged


def read_track(path):
    """Snapshots of a binary track file: list of (time, planets, particles)
    with planets / particles as TRACK_RECORD arrays."""
    data = open(path, "rb").read()
    out = []
    pos = 0
    while pos < len(data):
        (t,) = struct.unpack_from("<d", data, pos)
        (npl,) = struct.unpack_from("<Q", data, pos + 8)
        pos += 16
        pl = np.frombuffer(data, TRACK_RECORD, npl, pos)
        pos += npl * TRACK_RECORD.itemsize
        (npa,) = struct.unpack_from("<Q", data, pos)
        pos += 8
        pa = np.frombuffer(data, TRACK_RECORD, npa, pos)
        pos += npa * TRACK_RECORD.itemsize
        out.append((t, pl, pa))
    return out


def merge_tracks(paths, out_path):
    """Merges per-rank track files (same snapshots, disjoint particle ids)
    into one file in the single-process layout: planets from the first
    rank, particle records of all ranks ordered by id.  Returns the number
    of snapshots."""
    per_rank = [read_track(p) for p in paths]
    n = len(per_rank[0])
    if any(len(s) != n for s in per_rank):
        raise ValueError("track files hold different numbers of snapshots")
    with open(out_path, "wb") as f:
        for k in range(n):
            t, pl, _ = per_rank[0][k]
            if any(s[k][0] != t for s in per_rank):
                raise ValueError("snapshot %d: ranks disagree on the time" % k)
            pa = np.concatenate([s[k][2] for s in per_rank])
            pa = pa[np.argsort(pa["id"], kind="stable")]
            f.write(struct.pack("<dQ", t, len(pl)))
            f.write(pl.tobytes())
            f.write(struct.pack("<Q", len(pa)))
            f.write(pa.tobytes())
    return n
