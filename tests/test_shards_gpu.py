"""Several ranks over one file, each rank's work on the GPU (summaries and
seeded passes run in turn on this GPU; the exchange is the host logic of
the sharded path): concatenation == whole-file index and tape, and every
GPU summary == the oracle's."""

import numpy as np
import pytest

import oracle
from falx_gb300 import gen, shards
from shard_oracle import OracleShards, cut_points
from test_shards import CASES, run_world

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,dialect", CASES)
def test_gpu_ranks(engine, kind, dialect):
    doc = bytes(gen.generate(kind, 6 << 20))
    want_i = oracle.index_spec(doc, dialect)
    want_s, want_e = oracle.parse_tape(doc, dialect)
    rng = np.random.default_rng(100 + kind)
    gpu = shards.GpuShards(engine)
    for world in (2, 3, 4):
        bounds = cut_points(len(doc), rng, world)
        for lo, hi in bounds:
            prev = doc[lo - 1] if lo else -1
            g = gpu.summary(doc[lo:hi], dialect, prev)
            o = OracleShards().summary(doc[lo:hi], dialect, prev)
            for k in ("exit", "structurals", "terminators", "rows"):
                assert g[k] == o[k], (k, lo, hi)
        idx, seps, ends = run_world(doc, dialect, bounds, gpu)
        assert np.array_equal(idx.view(np.uint32), want_i), (world, bounds)
        assert np.array_equal(seps.view(np.uint32), want_s)
        assert np.array_equal(ends.view(np.uint64), want_e)


def test_gpu_seams(engine):
    doc = b'a,"x\n#y",b\n#c,"d\n"e,f\n"g\\\\"h\n' * 3000
    gpu = shards.GpuShards(engine)
    for dialect in (0, 1, 3, 4):
        want = oracle.index_spec(doc, dialect)
        for step in (1, 5, 16383, 16385, 40000):
            bounds = [(i, min(i + step, len(doc))) for i in range(0, len(doc), step)][:12]
            bounds[-1] = (bounds[-1][0], len(doc))
            idx, _, _ = run_world(doc, dialect, bounds, gpu)
            assert np.array_equal(idx.view(np.uint32), want), (dialect, step)


@pytest.mark.parametrize("kind,dialect,columns", [(gen.CSV_HASH, 1, [(0, 1), (1, 3), (3, 1), (4, 2), (5, 2), (2, 4)]),
                                                   (gen.CSV_GEO, 0, [(1, 3), (4, 2), (5, 2)]),
                                                   (gen.ADVERSARIAL, 1, [(0, 3), (1, 4), (2, 2)]),
                                                   (gen.LOGFMT, 3, [(0, 3), (1, 3), (3, 4)])])
def test_gpu_ranks_columns(engine, kind, dialect, columns):
    """Sharded typed columns (each rank's part parsed on the GPU, joined on
    the host) == the single-GPU columns == the oracle's."""
    import falx_gb300 as fx
    from shard_oracle import sharded_columns
    from test_shards import assert_table

    doc = bytes(gen.generate(kind, 6 << 20))
    want = oracle.parse_columns(doc, dialect, columns)
    single = engine.parse_columns(doc, fx.Schema(dialect, columns))
    assert_table((single.rows, [single.host(k) for k in range(len(columns))]), want, columns, "single")
    rng = np.random.default_rng(300 + kind)
    for world in (2, 3, 8):
        bounds = cut_points(len(doc), rng, world)
        got = sharded_columns(doc, dialect, columns, bounds, shards.GpuShards(engine))
        assert_table(got, want, columns, (world, bounds))


def test_gpu_columns_seams(engine):
    from shard_oracle import sharded_columns
    from test_shards import assert_table

    doc = b'a,"x\n#y",b\n#c,"d\n"e,f\n"g\\\\"h\n1,"2""3",4\n' * 2000 + b'last,"open'
    cols = [(0, 3), (1, 3), (2, 4)]
    for dialect in (0, 1, 3):
        want = oracle.parse_columns(doc, dialect, cols)
        for step in (1, 7, 16385, 40000):
            bounds = [(i, min(i + step, len(doc))) for i in range(0, len(doc), step)][:10]
            bounds[-1] = (bounds[-1][0], len(doc))
            got = sharded_columns(doc, dialect, cols, bounds, shards.GpuShards(engine))
            assert_table(got, want, cols, (dialect, step))


def _gpu_rank(rank, world, port, path):
    """One rank of a gloo world on this GPU: summaries and counts go through
    gloo, the rank's summary, seeded passes and column part run on the GPU."""
    import os

    import torch.distributed as dist

    import falx_gb300 as fx

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    eng = fx.Engine(0)
    gpu = shards.GpuShards(eng)
    doc = bytes(gen.generate(gen.CSV_HASH, 8 << 20))
    cols = [(0, 1), (1, 3), (4, 2)]
    lo, hi = shards.shard_bounds(len(doc), world)[rank]
    prev = doc[lo - 1] if lo else -1
    res = shards.parse_sharded(gpu, doc[lo:hi], 1, rank, lo, prev, shards.torch_all_gather)
    part = shards.parse_columns_sharded(gpu, doc[lo:hi], 1, cols, rank, lo, prev, len(doc), lambda a, b: doc[a:b],
                                        shards.torch_all_gather)
    tape = {k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in res.items()}
    rows, host = gpu.part_host(part["columns"], cols)
    parts = shards.torch_all_gather((tape, (rows, host, part["pos_at"])))
    if rank == 0:
        idx, seps, ends = shards.assemble([p[0] for p in parts])
        table = shards.assemble_columns([p[1] for p in parts], cols)
        s, e = oracle.parse_tape(doc, 1)
        want_rows, want_cols = oracle.parse_columns(doc, 1, cols)
        ok = (np.array_equal(idx.view(np.uint32), oracle.index_spec(doc, 1)) and
              np.array_equal(seps.view(np.uint32), s) and np.array_equal(ends.view(np.uint64), e) and
              table[0] == want_rows and
              np.array_equal(table[1][0]["values"].view(np.uint32), want_cols[0]["values"]) and
              table[1][1]["data"] == want_cols[1]["data"] and
              np.array_equal(table[1][1]["offsets"], want_cols[1]["offsets"]) and
              np.array_equal(table[1][2]["values"].view(np.uint64), want_cols[2]["values"].view(np.uint64)) and
              all(np.array_equal(table[1][k]["valid"], want_cols[k]["valid"]) for k in range(3)))
        with open(path, "w") as f:
            f.write("ok" if ok else "mismatch")
    dist.barrier()
    eng.close()
    dist.destroy_process_group()


def test_gloo_two_ranks_on_gpu(tmp_path):
    """World size 2 over gloo, each rank driving GpuShards on this GPU (the
    ranks never wait on each other's kernels; they meet only on the host)."""
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    path = str(tmp_path / "result")
    mp.spawn(_gpu_rank, args=(2, port, path), nprocs=2, join=True)
    assert open(path).read() == "ok"
