"""Batched documents on the GPU (falx_batch_*): each document's structural
index and lat / lon f64 columns against the oracle, for every staging depth
and chunk size, across graph replays, and after autotuning."""

import numpy as np
import pytest

import falx_gb300 as fx
import oracle
from falx_gb300 import batch

pytestmark = pytest.mark.gpu


def make(engine, ndocs=90, total=24 << 20, seed=1):
    import torch

    sizes = batch.mixed_sizes(ndocs, total, lo=1 << 10, hi=8 << 20, seed=seed)
    sizes[:4] = [0, 1, 37, 16384]  # empty, one byte, tiny, one exact tile
    dialects = batch.mixed_dialects(ndocs, seed=seed + 1)
    host, offs, lens = batch.generate(sizes, dialects, seed=seed + 100)
    # one document cut mid-record and one ending without a newline
    lens[5] = max(lens[5] - 7, 0)
    data = torch.from_numpy(host).cuda()
    return host, offs, lens, dialects, data


def check_docs(b, host, offs, lens, dialects, which=None):
    for k in which if which is not None else range(len(lens)):
        doc = host[offs[k]: offs[k] + lens[k]].tobytes()
        d = int(dialects[k])
        assert b.docs[k].status == 0, k
        idx, c0, v0, c1, v1 = b.result(k)
        assert np.array_equal(idx, oracle.index_spec(doc, d)), ("index", k, d)
        f0, f1 = batch.GEO_FIELDS[d]
        rows, want = oracle.parse_columns(doc, d, [(f0, fx.F64), (f1, fx.F64)])
        assert b.docs[k].rows == rows, ("rows", k)
        assert np.array_equal(c0.view(np.uint64), np.asarray(want[0]["values"]).view(np.uint64)), ("col0", k)
        assert np.array_equal(c1.view(np.uint64), np.asarray(want[1]["values"]).view(np.uint64)), ("col1", k)
        assert np.array_equal(v0, want[0]["valid"]), ("valid0", k)
        assert np.array_equal(v1, want[1]["valid"]), ("valid1", k)


@pytest.mark.parametrize("config", [(64 << 10, 0, 2), (1 << 20, 0, 3), (4 << 20, 1, 2), (256 << 10, 2, 3)])
def test_batch_matches_oracle(engine, config):
    host, offs, lens, dialects, data = make(engine)
    b = batch.Batch(engine, data, offs, lens, dialects, config=config)
    b.run()
    check_docs(b, host, offs, lens, dialects)
    info = b.info()
    assert info["staging"] == config[2] and info["chunk_bytes"] == config[0]
    # a second replay of the same plan gives the same outputs
    b.run()
    check_docs(b, host, offs, lens, dialects, which=range(0, len(lens), 7))
    b.close()


def test_batch_tuned(engine):
    host, offs, lens, dialects, data = make(engine, ndocs=60, total=16 << 20, seed=9)
    b = batch.Batch(engine, data, offs, lens, dialects)
    best = batch.tune(engine, b)
    assert best["staging"] in (2, 3) and best["chunk_bytes"] in (64 << 10, 256 << 10, 1 << 20, 4 << 20)
    b.close()
    b = batch.Batch(engine, data, offs, lens, dialects)  # planned with the tuned configuration
    info = b.info()
    assert (info["chunk_bytes"], info["staging"]) == (best["chunk_bytes"], best["staging"])
    b.run()
    check_docs(b, host, offs, lens, dialects)
    b.close()


def test_batch_capacity_is_per_document(engine):
    import torch

    from falx_gb300 import _lib

    host, offs, lens, dialects, data = make(engine, ndocs=8, total=2 << 20, seed=5)
    b = batch.Batch(engine, data, offs, lens, dialects, config=(1 << 20, 0, 2))
    b.docs[6].index_cap = 3  # too small for document 6 only
    b.close()
    ptr = __import__("ctypes").c_void_p()
    assert engine.lib.falx_batch_create(engine.ctx, b.docs, b.n, None, __import__("ctypes").byref(ptr)) == 0
    rc = engine.lib.falx_batch_run(ptr, b.docs)
    assert rc == _lib.FALX_ERR_CAPACITY
    assert b.docs[6].status == _lib.FALX_ERR_CAPACITY and b.docs[6].n_index > 3
    assert all(b.docs[k].status == 0 for k in range(8) if k != 6)
    engine.lib.falx_batch_destroy(ptr)
