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

Typed columns (parse_columns_sharded) assign records by their start, as
parse_columns_chunks_par does (csv_hash.rs:1499-1557: a worker skips to the
first record boundary at or past its chunk start and finishes the record it
is in at the chunk end). After the summary fold every rank knows its entry
state, finds the first record start in its shard (a seeded pass over a short
window at the shard start), and the ranks exchange those starts. Rank r then
parses its records [S_r, S_r+1) as one document: a record start is a clean
state of every dialect's automaton (outside any region, at a line start), so
the parts concatenate to the whole file's columns. The bytes of the last
record past the shard end are read from the file (`read(lo, hi)`), as the
reference's workers read past their chunk. A second exchange of row and
string-arena counts places every part in the global table (row_at,
arena_at); assemble_columns joins parts into one table, rebasing string
offsets and spans and shifting validity bitmaps across the seams
(parse_columns_par, csv_hash.rs:1559-1660).
"""

from ctypes import byref, c_uint64, c_void_p

import numpy as np

from . import _lib
from ._lib import BYTES, STR, check


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
    """The GPU side of a rank: summary and seeded pass on this engine.
    With full=True a part's parse also produces its structural index, tape
    and field-byte totals (one falx_parse pass), kept in `last`."""

    def __init__(self, engine, full=False):
        self.engine = engine
        self.full = full
        self.last = None

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


    def first_terminator(self, shard, dialect, prev_byte, entry, window=64 << 10):
        """Offset of the first terminator in the shard under entry state
        `entry`, or None: seeded passes over a window at the shard start,
        grown until it holds a terminator or the whole shard."""
        e = self.engine
        torch = e.torch
        d = e.to_device(shard)
        e._sync_stream()
        n = d.numel()
        ends = e.empty(16, torch.int64)
        w = window
        while True:
            m = min(w, n)
            a, b, c = c_uint64(), c_uint64(), c_uint64()
            rc = e.lib.falx_parse_tape_seeded(e.ctx, dialect, c_void_p(d.data_ptr()), m, prev_byte, entry, 0, 0, None,
                                              0, None, 0, c_void_p(ends.data_ptr()), 16, byref(a), byref(b), byref(c))
            if rc != _lib.FALX_ERR_CAPACITY:
                check(rc, "falx_parse_tape_seeded")
            if c.value:
                return int(ends[0].item()) & 0xFFFFFFFF
            if m == n:
                return None
            w *= 4

    def make_piece(self, shard, a, b, tail):
        """The part's bytes on this GPU: shard[a:b] followed by `tail` (host
        bytes from past the shard). A device shard that is a view with room
        after it in its buffer takes the tail in place."""
        e = self.engine
        torch = e.torch
        d = e.to_device(shard)
        if not len(tail):
            return d[a:b]
        t = torch.from_numpy(np.frombuffer(bytes(tail), dtype=np.uint8).copy())
        room = d.untyped_storage().nbytes() - d.storage_offset() - d.numel()
        if d.is_cuda and b == d.numel() and room >= t.numel():
            full = torch.empty(0, dtype=torch.uint8, device=d.device)
            full.set_(d.untyped_storage(), d.storage_offset(), (d.numel() + t.numel(),))
            full[d.numel():].copy_(t, non_blocking=False)
            return full[a:]
        return torch.cat([d[a:b], t.to(d.device)])

    def columns(self, piece, dialect, columns):
        """Typed columns of one part (a run of whole records) on this GPU."""
        from . import Schema

        if self.full:
            self.last = self.engine.parse_all(piece, Schema(dialect, columns), stats_fields=None)
            return self.last["columns"]
        return self.engine.parse_columns(piece, Schema(dialect, columns))

    @staticmethod
    def part_host(part, columns):
        return part.rows, [part.host(k) for k in range(len(columns))]


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


def fixed_all_gather(obj, device, nbytes=2048):
    """all_gather of a small picklable object in one collective: the pickle
    padded to `nbytes` in a uint8 tensor on `device` (NCCL needs a CUDA
    device, gloo takes CPU)."""
    import pickle

    import torch
    import torch.distributed as dist

    raw = pickle.dumps(obj)
    if len(raw) + 4 > nbytes:
        return torch_all_gather(obj)
    buf = np.zeros(nbytes, dtype=np.uint8)
    buf[:4] = np.frombuffer(np.uint32(len(raw)).tobytes(), dtype=np.uint8)
    buf[4: 4 + len(raw)] = np.frombuffer(raw, dtype=np.uint8)
    mine = torch.from_numpy(buf).to(device)
    world = dist.get_world_size()
    out = torch.empty(world * nbytes, dtype=torch.uint8, device=device)
    dist.all_gather_into_tensor(out, mine)
    host = out.cpu().numpy().reshape(world, nbytes)
    res = []
    for r in range(world):
        n = int(host[r, :4].view(np.uint32)[0])
        res.append(pickle.loads(host[r, 4: 4 + n].tobytes()))
    return res


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


def record_start(backend, shard, dialect, prev_byte, entry, summary):
    """Offset of the first record start in the shard, or None. The shard's
    first byte starts a record at the file start or right after a newline
    that left the automaton in its initial state (a structural newline:
    inside a quote or an escape the state would differ)."""
    if len(shard) == 0:
        return None
    if prev_byte < 0 or (prev_byte == 0x0A and entry == 0):
        return 0
    if summary["terminators"][entry] == 0:
        return None
    t = backend.first_terminator(shard, dialect, prev_byte, entry)
    return t + 1 if t is not None and t + 1 < len(shard) else None


def resolve_starts(starts, n):
    """Part bounds from every rank's first record start (file offsets or
    None): a rank without one owns no records."""
    bounds = [n] * (len(starts) + 1)
    for r in range(len(starts) - 1, -1, -1):
        bounds[r] = starts[r] if starts[r] is not None else bounds[r + 1]
    return bounds


def parse_columns_sharded(backend, shard, dialect, columns, rank, pos_base, prev_byte, file_len, read, all_gather):
    """One rank's part of the whole file's typed columns.

    `shard` holds the file's bytes [pos_base, pos_base + len(shard));
    `read(lo, hi)` returns any other range of the file (the part's last
    record may run past the shard); `all_gather(obj)` returns every rank's
    obj in rank order. Returns dict(columns: the part's columns in its own
    frame, rows, row_at, arena_at (per column), pos_at: the part's file
    offset, bounds: (start, end) of the part)."""
    mine = backend.summary(shard, dialect, prev_byte)
    summaries = all_gather(mine)
    entry, _, _, _ = fold(summaries, rank)
    st = record_start(backend, shard, dialect, prev_byte, entry, mine)
    starts = all_gather(None if st is None else pos_base + st)
    bounds = resolve_starts(starts, file_len)
    lo, hi = bounds[rank], bounds[rank + 1]
    end = pos_base + len(shard)
    if lo >= hi:
        piece = backend.make_piece(shard, 0, 0, b"")
    elif hi <= end:
        piece = backend.make_piece(shard, lo - pos_base, hi - pos_base, b"")
    else:
        piece = backend.make_piece(shard, lo - pos_base, len(shard), read(end, hi))
    part = backend.columns(piece, dialect, columns)
    rows = part.rows if hasattr(part, "rows") else part[0]
    lens = _str_lens(part, columns)
    counts = all_gather((rows, lens))
    row_at = sum(c[0] for c in counts[:rank])
    arena_at = [sum(c[1][k] for c in counts[:rank]) for k in range(len(columns))]
    return {"columns": part, "rows": rows, "row_at": row_at, "arena_at": arena_at, "pos_at": lo,
            "bounds": (lo, hi)}


def _str_lens(part, columns):
    if hasattr(part, "_str_lens"):
        return [int(x) for x in part._str_lens]
    return [len(c["data"]) if "data" in c else 0 for c in part[1]]


def assemble_columns(parts, columns):
    """Join per-rank parts, given as (rows, host column dicts, pos_at) in
    rank order, into one table in the oracle's host layout: (rows, [per
    column dict]). String offsets continue across parts, (from, to) spans
    get the part's file offset, validity bitmaps shift to the part's first
    row."""
    total = sum(p[0] for p in parts)
    out = []
    for k, (f, t) in enumerate(columns):
        bits = []
        vals, offs, arena, spans = [], [np.zeros(1, np.int32)], [], []
        base = 0
        for rows, cols, pos_at in parts:
            c = cols[k]
            v = np.unpackbits(np.asarray(c["valid"], dtype=np.uint64).view(np.uint8), bitorder="little")[:rows]
            bits.append(v)
            if "offsets" in c:
                offs.append(np.asarray(c["offsets"][1: rows + 1], dtype=np.int64) + base)
                arena.append(bytes(c["data"]))
                base += len(c["data"])
            elif "spans" in c:
                sp = np.asarray(c["spans"], dtype=np.uint64).reshape(-1, 2)[:rows].copy()
                sp[v.astype(bool)] += np.uint64(pos_at)
                spans.append(sp.astype(np.uint32))
            else:
                vals.append(np.asarray(c["values"])[:rows])
        b = np.concatenate(bits) if bits else np.zeros(0, np.uint8)
        words = (total + 63) // 64
        packed = np.zeros(words * 8, np.uint8)
        pb = np.packbits(b, bitorder="little")
        packed[: pb.size] = pb
        col = {"valid": packed.view(np.uint64)}
        if t == STR:
            col["offsets"] = np.concatenate(offs).astype(np.int32)
            col["data"] = b"".join(arena)
        elif t == BYTES:
            col["spans"] = np.concatenate(spans) if spans else np.zeros((0, 2), np.uint32)
        else:
            col["values"] = np.concatenate(vals) if vals else np.zeros(0)
        out.append(col)
    return total, out
