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


def cut_points(n, rng, world):
    """Shard boundaries: some equal, some random."""
    if rng.random() < 0.5:
        return [(n * r // world, n * (r + 1) // world) for r in range(world)]
    cuts = sorted(set([0, n] + [int(x) for x in rng.integers(0, n + 1, world - 1)]))
    while len(cuts) < world + 1:
        cuts.append(n)
    return list(zip(cuts[:-1], cuts[1:]))
