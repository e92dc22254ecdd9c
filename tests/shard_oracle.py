"""CPU stand-in for a rank's GPU work in the sharded tests: summary and
seeded pass from the oracle's serial restatement (test infrastructure)."""

import numpy as np

import oracle


class OracleShards:
    def summary(self, shard, dialect, prev_byte):
        per = oracle.shard_summary(shard, dialect, prev_byte)
        return {"exit": [p["exit"] for p in per], "structurals": [p["structurals"] for p in per],
                "terminators": [p["terminators"] for p in per], "rows": [p["rows"] for p in per],
                "last_byte": shard[-1] if len(shard) else -1}

    def tape_seeded(self, shard, dialect, prev_byte, entry, pos_base, sep_base, counts):
        idx, _, _, _ = oracle.index_seeded(shard, dialect, entry, prev_byte, pos_base)
        raw = np.frombuffer(bytes(shard), dtype=np.uint8)
        is_nl = raw[idx.astype(np.int64) - pos_base] == 0x0A if idx.size else np.zeros(0, bool)
        seps = idx[~is_nl]
        sep_before = sep_base + np.cumsum(~is_nl) - (~is_nl)  # separators before each structural
        ends = (sep_before[is_nl].astype(np.uint64) << np.uint64(32)) | idx[is_nl].astype(np.uint64)
        return idx, seps, ends


    def first_terminator(self, shard, dialect, prev_byte, entry):
        idx, _, _, _ = oracle.index_seeded(shard, dialect, entry, prev_byte, 0)
        raw = np.frombuffer(bytes(shard), dtype=np.uint8)
        nl = idx[raw[idx.astype(np.int64)] == 0x0A] if idx.size else idx
        return int(nl[0]) if nl.size else None

    @staticmethod
    def make_piece(shard, a, b, tail):
        return bytes(shard[a:b]) + bytes(tail)

    def columns(self, piece, dialect, columns):
        return oracle.parse_columns(piece, dialect, columns)

    @staticmethod
    def part_host(part, columns):
        return part


class ThreadWorld:
    """Ranks as threads of one process: all_gather through a barrier, and
    one lock around every backend call (ranks on one GPU run in turn)."""

    def __init__(self, world):
        import threading

        self.world = world
        self.slots = [None] * world
        self.barrier = threading.Barrier(world)
        self.lock = threading.Lock()

    def gather_for(self, rank):
        def gather(obj):
            self.slots[rank] = obj
            self.barrier.wait()
            out = list(self.slots)
            self.barrier.wait()
            return out
        return gather

    def locked(self, backend):
        world = self

        class Locked:
            def __getattr__(self, name):
                fn = getattr(backend, name)

                def call(*a, **k):
                    with world.lock:
                        return fn(*a, **k)
                return call
        return Locked()

    def run(self, fn):
        """fn(rank, gather) on every rank; results in rank order."""
        import threading

        out, errs = [None] * self.world, []

        def body(r):
            try:
                out[r] = fn(r, self.gather_for(r))
            except BaseException as e:  # noqa: BLE001 - re-raised below
                errs.append(e)
                self.barrier.abort()

        ts = [threading.Thread(target=body, args=(r,)) for r in range(self.world)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        if errs:
            raise errs[0]
        return out


def sharded_columns(doc, dialect, columns, bounds, backend):
    """Every rank's parse_columns_sharded over `bounds`, joined into one
    host table (rows, columns)."""
    from falx_gb300 import shards

    world = ThreadWorld(len(bounds))
    be = world.locked(backend)

    def rank(r, gather):
        lo, hi = bounds[r]
        res = shards.parse_columns_sharded(be, doc[lo:hi], dialect, columns, r, lo, doc[lo - 1] if lo else -1,
                                           len(doc), lambda a, b: doc[a:b], gather)
        rows, host = backend.part_host(res["columns"], columns)
        return res, (rows, host, res["pos_at"])

    out = world.run(rank)
    for (p, _), (q, _) in zip(out, out[1:]):
        assert p["row_at"] + p["rows"] == q["row_at"] and p["bounds"][1] == q["bounds"][0]
    return shards.assemble_columns([x[1] for x in out], columns)


def cut_points(n, rng, world):
    """Shard boundaries: some equal, some random."""
    if rng.random() < 0.5:
        return [(n * r // world, n * (r + 1) // world) for r in range(world)]
    cuts = sorted(set([0, n] + [int(x) for x in rng.integers(0, n + 1, world - 1)]))
    while len(cuts) < world + 1:
        cuts.append(n)
    return list(zip(cuts[:-1], cuts[1:]))
