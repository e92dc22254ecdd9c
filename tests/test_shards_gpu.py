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
