"""Several ranks over one file (host logic): summaries exchanged, folded
into entry states and offsets, seeded passes concatenated == the whole-file
serial index and tape. Ranks are gloo processes (world size 2) and a
simulated world of up to 5 in one process; the per-rank work is the oracle."""

import os
import socket

import numpy as np
import pytest

import oracle
from falx_gb300 import gen, shards
from shard_oracle import OracleShards, cut_points

CASES = [(gen.ADVERSARIAL, 1), (gen.CSV_GEO, 0), (gen.LOGFMT, 3), (gen.NDJSON, 4), (gen.TSV, 2)]


def run_world(doc, dialect, bounds, backend):
    parts = []
    local = []

    def gather(obj):
        local.append(obj)
        return local

    # simulated all-gather: every rank's summary first, then the seeded passes
    summaries = [backend.summary(doc[lo:hi], dialect, doc[lo - 1] if lo else -1) for lo, hi in bounds]
    for r, (lo, hi) in enumerate(bounds):
        res = shards.parse_sharded(backend, doc[lo:hi], dialect, r, lo, doc[lo - 1] if lo else -1,
                                   lambda obj: summaries)
        parts.append({k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in res.items()})
    for p, q in zip(parts, parts[1:]):
        assert p["index_at"] + len(p["index"]) == q["index_at"]
    return shards.assemble(parts)


@pytest.mark.parametrize("kind,dialect", CASES)
def test_simulated_world(kind, dialect):
    doc = bytes(gen.generate(kind, 1 << 20))
    want_i = oracle.index_spec(doc, dialect)
    want_s, want_e = oracle.parse_tape(doc, dialect)
    rng = np.random.default_rng(kind * 7 + dialect)
    for world in (1, 2, 3, 5):
        for _ in range(3):
            bounds = cut_points(len(doc), rng, world)
            idx, seps, ends = run_world(doc, dialect, bounds, OracleShards())
            assert np.array_equal(idx.astype(np.uint32), want_i), (world, bounds)
            assert np.array_equal(seps.astype(np.uint32), want_s)
            assert np.array_equal(ends.astype(np.uint64), want_e)


def test_fold_hazards():
    # seams inside quotes, comments, escapes, right after '\n', 1-byte and empty shards
    doc = b'a,"x\n#y",b\n#c,"d\n"e,f\n"g\\\\"h\n' * 50
    for dialect in (0, 1, 3, 4):
        want = oracle.index_spec(doc, dialect)
        for step in (1, 2, 3, 7, 13):
            bounds = [(i, min(i + step, len(doc))) for i in range(0, len(doc), step)][:40]
            bounds[-1] = (bounds[-1][0], len(doc))
            bounds.insert(3, (bounds[2][1], bounds[2][1]))  # an empty shard
            idx, _, _ = run_world(doc, dialect, bounds, OracleShards())
            assert np.array_equal(idx.astype(np.uint32), want), (dialect, step)


def _rank(rank, world, port, path):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    doc = bytes(gen.generate(gen.ADVERSARIAL, 2 << 20))
    lo, hi = shards.shard_bounds(len(doc), world)[rank]
    res = shards.parse_sharded(OracleShards(), doc[lo:hi], 1, rank, lo, doc[lo - 1] if lo else -1,
                               shards.torch_all_gather)
    parts = shards.torch_all_gather({k: v for k, v in res.items()})
    if rank == 0:
        idx, seps, ends = shards.assemble(parts)
        s, e = oracle.parse_tape(doc, 1)
        ok = (np.array_equal(idx.astype(np.uint32), oracle.index_spec(doc, 1)) and
              np.array_equal(seps.astype(np.uint32), s) and np.array_equal(ends.astype(np.uint64), e))
        with open(path, "w") as f:
            f.write("ok" if ok else "mismatch")
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks(tmp_path):
    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    path = str(tmp_path / "result")
    mp.spawn(_rank, args=(2, port, path), nprocs=2, join=True)
    assert open(path).read() == "ok"


def _rank_fails(rank, world, port, path):
    import datetime

    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=5))
    if rank == 1:
        os._exit(3)  # the rank dies before the summary exchange
    doc = bytes(gen.generate(gen.CSV_HASH, 64 << 10))
    lo, hi = shards.shard_bounds(len(doc), world)[rank]
    try:
        shards.parse_sharded(OracleShards(), doc[lo:hi], 1, rank, lo, -1, shards.torch_all_gather)
        outcome = "no error"
    except Exception as e:  # the exchange fails instead of hanging
        outcome = "detected: " + type(e).__name__
    with open(path, "w") as f:
        f.write(outcome)
    os._exit(0)


def test_gloo_rank_failure_is_detected(tmp_path):
    # A rank that dies before the exchange: the surviving rank's all-gather
    # ends with an error (peer gone or the process-group timeout), never a
    # hang, and no GPU work of it is in flight.
    import time

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    path = str(tmp_path / "result")
    ctx = mp.spawn(_rank_fails, args=(2, port, path), nprocs=2, join=False)
    t0 = time.time()
    for p in ctx.processes:
        p.join(timeout=60)
    alive = [p for p in ctx.processes if p.is_alive()]
    for p in alive:
        p.kill()
    assert not alive, "a rank hung"
    assert time.time() - t0 < 60
    assert open(path).read().startswith("detected")


COL_CASES = [(gen.CSV_HASH, 1, [(0, 1), (1, 3), (3, 1), (4, 2), (5, 2), (2, 4)]),
             (gen.CSV_GEO, 0, [(1, 3), (4, 2), (5, 2), (0, 0)]),
             (gen.ADVERSARIAL, 1, [(0, 3), (1, 4), (2, 2)]),
             (gen.TSV, 2, [(0, 3), (1, 0), (2, 4)]),
             (gen.LOGFMT, 3, [(0, 3), (1, 3), (3, 4)])]


def assert_table(got, want, columns, ctx):
    rows, cols = got
    wrows, wcols = want
    assert rows == wrows, ctx
    for k, (f, t) in enumerate(columns):
        g, w = cols[k], wcols[k]
        assert np.array_equal(g["valid"][: (rows + 63) // 64], w["valid"][: (rows + 63) // 64]), (ctx, k)
        if t == 3:
            assert np.array_equal(g["offsets"], w["offsets"]) and g["data"] == w["data"], (ctx, k)
        elif t == 4:
            assert np.array_equal(np.asarray(g["spans"]).reshape(-1, 2), np.asarray(w["spans"]).reshape(-1, 2)), (ctx, k)
        else:
            assert np.array_equal(np.asarray(g["values"]).view(np.uint8), np.asarray(w["values"]).view(np.uint8)), \
                (ctx, k)


@pytest.mark.parametrize("kind,dialect,columns", COL_CASES)
def test_simulated_world_columns(kind, dialect, columns):
    from shard_oracle import sharded_columns

    doc = bytes(gen.generate(kind, 256 << 10))
    want = oracle.parse_columns(doc, dialect, columns)
    rng = np.random.default_rng(kind * 11 + dialect)
    for world in (1, 2, 3, 5):
        for _ in range(3):
            bounds = cut_points(len(doc), rng, world)
            got = sharded_columns(doc, dialect, columns, bounds, OracleShards())
            assert_table(got, want, columns, (world, bounds))


def test_columns_seams():
    # seams inside quotes, comments, escapes, right after '\n', 1-byte and
    # empty shards, shards without a record start, a file without a final newline
    from shard_oracle import sharded_columns

    doc = b'a,"x\n#y",b\n#c,"d\n"e,f\n"g\\\\"h\n1,"2""3",4\n' * 40 + b'last,"open'
    for dialect in (0, 1, 3):
        cols = [(0, 3), (1, 3), (2, 4)]
        want = oracle.parse_columns(doc, dialect, cols)
        for step in (1, 2, 3, 7, 13, 101):
            bounds = [(i, min(i + step, len(doc))) for i in range(0, len(doc), step)][:30]
            bounds[-1] = (bounds[-1][0], len(doc))
            bounds.insert(3, (bounds[2][1], bounds[2][1]))
            got = sharded_columns(doc, dialect, cols, bounds, OracleShards())
            assert_table(got, want, cols, (dialect, step))
