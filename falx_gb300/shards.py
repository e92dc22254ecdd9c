"""One file over several GPUs: contiguous shards, one per rank.

Each rank (one process per GPU):
  1. summarises its shard for every possible entry state
     (falx_summarize_shard: exit state and structural / terminator / row
     counts per entry state, from local passes only);
  2. exchanges the summaries with every other rank (an all-gather of a few
     dozen bytes per rank, through the host: torch.distributed with gloo or
     NCCL, or any all-gather callable);
  3. folds the summaries of the ranks before it into its true entry state
     and output offsets (an exclusive scan of the transfer functions);
  4. runs a seeded pass that writes its part of the global structural index
     and tape (falx_parse_tape_seeded), with file positions and separator
     counts continued from the ranks before it.

The byte before a shard decides whether the shard starts a line and a
record; the caller passes it (ranks read their shard plus that byte).
This follows the reference's three-phase parallel drivers (csv_hash.rs
:152-214 region transfer functions per chunk, serial compose, seeded pass;
csv_geo.rs:95-149) with ranks in place of threads. Records that cross a shard
seam belong to the shard holding their terminator, as in the reference's
chunked drivers: the tape of rank r ends at its last terminator and the next
rank's separators continue that record's count.
"""

from ctypes import byref, c_uint64, c_void_p

import numpy as np

from . import _lib
from ._lib import check


def shard_bounds(n, world):
    """Contiguous byte ranges [(lo, hi)] of nearly equal size."""
    return [(n * r // world, n * (r + 1) // world) for r in range(world)]


def fold(summaries, rank):
    """Entry state and counts before shard `rank`: (state, structurals,
    terminators, rows)."""
    state, s, t, r = 0, 0, 0, 0
    for sm in summaries[:rank]:
        s += sm["structurals"][state]
        t += sm["terminators"][state]
        r += sm["rows"][state]
        state = sm["exit"][state]
    return state, s, t, r


class GpuShards:
    """The GPU side of a rank: summary and seeded pass on this engine."""

    def __init__(self, engine):
        self.engine = engine

    def summary(self, shard, dialect, prev_byte):
        e = self.engine
        d = e.to_device(shard)
        e._sync_stream()
        out = _lib.falx_shard_summary()
        check(e.lib.falx_summarize_shard(e.ctx, dialect, c_void_p(d.data_ptr()), d.numel(), prev_byte, byref(out)),
              "falx_summarize_shard")
        n = out.states
        return {"exit": list(out.exit)[:n], "structurals": list(out.structurals)[:n],
                "terminators": list(out.terminators)[:n], "rows": list(out.rows)[:n], "last_byte": out.last_byte}

    def tape_seeded(self, shard, dialect, prev_byte, entry, pos_base, sep_base, counts):
        """(index, seps, ends) of the shard as part of the file; `counts` =
        (structurals, terminators) the summary gave for this entry."""
        e = self.engine
        torch = e.torch
        d = e.to_device(shard)
        e._sync_stream()
        ns, nt = counts
        index = e.empty(max(ns, 1), torch.int32)
        seps = e.empty(max(ns - nt, 1), torch.int32)
        ends = e.empty(max(nt, 1), torch.int64)
        a, b, c = c_uint64(), c_uint64(), c_uint64()
        check(e.lib.falx_parse_tape_seeded(e.ctx, dialect, c_void_p(d.data_ptr()), d.numel(), prev_byte, entry,
                                           pos_base, sep_base, c_void_p(index.data_ptr()), max(ns, 1),
                                           c_void_p(seps.data_ptr()), max(ns - nt, 1), c_void_p(ends.data_ptr()),
                                           max(nt, 1), byref(a), byref(b), byref(c)), "falx_parse_tape_seeded")
        return index[: a.value], seps[: b.value], ends[: c.value]


def parse_sharded(backend, shard, dialect, rank, pos_base, prev_byte, all_gather):
    """One rank's part of the whole file's index and tape.

    `all_gather(obj)` returns the list of every rank's obj in rank order.
    Returns dict(index, seps, ends and their global start offsets)."""
    mine = backend.summary(shard, dialect, prev_byte)
    summaries = all_gather(mine)
    entry, s, t, _ = fold(summaries, rank)
    ns, nt = mine["structurals"][entry], mine["terminators"][entry]
    index, seps, ends = backend.tape_seeded(shard, dialect, prev_byte, entry, pos_base, s - t, (ns, nt))
    return {"entry": entry, "index": index, "index_at": s, "seps": seps, "seps_at": s - t, "ends": ends,
            "ends_at": t}


def torch_all_gather(obj):
    """all_gather through torch.distributed (gloo or NCCL process group)."""
    import torch.distributed as dist

    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out


def assemble(parts):
    """Concatenate per-rank outputs (host arrays) in rank order."""
    cat = lambda k: np.concatenate([np.asarray(p[k]) for p in parts]) if parts else np.zeros(0)
    return cat("index"), cat("seps"), cat("ends")
