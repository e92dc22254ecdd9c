"""Every benchmarked workload at its full size on the GPU, against the CPU
oracle on the same bytes (the parallel port of the reference's drivers):

  csv-geo 64 MiB      structural index, lat / lon f64 columns, count / sum
  csv_hash 1 GiB      structural index, field bytes, u32 / str / f64 columns
  NDJSON 1 GiB        records and sum(id + nested.score)
  adversarial 1 GiB   the speculative index equals the plain one and the oracle's
  batch of 4096 docs  (6 GiB) a seeded sample of documents, each against the oracle

Bit-for-bit except the f64 sums, which must lie within 1e-12 relative of
the oracle's sequential fold (csv_geo.rs:1735-1750 keeps bit checksums; the
exact fixed-point sums are compared exactly)."""

import os

import numpy as np
import pytest

import falx_gb300 as fx
import oracle
from falx_gb300 import gen

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
HASH_COLS = [(0, fx.U32), (1, fx.STR), (3, fx.U32), (4, fx.F64), (5, fx.F64)]


def assert_columns(got, want, cols):
    for k, (f, t) in enumerate(cols):
        h = got.host(k)
        assert np.array_equal(h["valid"], want[k]["valid"]), "validity of column %d" % k
        if t == fx.STR:
            assert np.array_equal(h["offsets"], want[k]["offsets"]), "offsets of column %d" % k
            assert h["data"] == want[k]["data"], "arena of column %d" % k
        else:
            assert np.array_equal(h["values"].view(np.uint8), want[k]["values"].view(np.uint8)), "column %d" % k


def test_csv_hash_1gib_step(engine):
    data = gen.generate(gen.CSV_HASH, 1 << 30)
    got = engine.parse_all(data, fx.Schema(fx.CSV_HASH, HASH_COLS))
    want = oracle.parse_par(data, oracle.CSV_HASH, HASH_COLS, THREADS)
    idx = got["index"].cpu().numpy().view(np.uint32)
    assert idx.size == want["index"].size and np.array_equal(idx, want["index"])
    assert (got["field_bytes"].fields, got["field_bytes"].bytes) == want["field_bytes"]
    assert got["columns"].rows == want["rows"]
    assert_columns(got["columns"], want["columns"], HASH_COLS)


def test_csv_geo_64mib_columns_and_stats(engine):
    data = gen.generate(gen.CSV_GEO, 64 << 20)
    cols = [(4, fx.F64), (5, fx.F64)]
    got = engine.parse_all(data, fx.Schema(fx.CSV, cols), stats_fields=(4, 5))
    want = oracle.parse_par(data, oracle.CSV, cols, THREADS, field_bytes=False, stats_fields=(4, 5))
    assert np.array_equal(got["index"].cpu().numpy().view(np.uint32), want["index"])
    assert got["columns"].rows == want["rows"]
    assert_columns(got["columns"], want["columns"], cols)
    st, ws = got["stats"], want["stats"]
    assert st.records == ws.records
    assert list(st.values) == list(ws.values) and list(st.checksum) == list(ws.checksum)
    assert list(st.sum_e6) == list(ws.sum_e6) and list(st.inexact) == list(ws.inexact)
    fold = oracle.geo_stats(data, oracle.CSV, 4, 5).fold  # sequential, row order
    for k in range(2):
        assert abs(st.sum_f64[k] - fold[k]) <= 1e-12 * max(1.0, abs(fold[k]))


def test_ndjson_1gib(engine):
    data = gen.generate(gen.NDJSON, 1 << 30)
    got = engine.ndjson_id_score(data)
    want = oracle.ndjson_json(data, threads=THREADS)
    assert got.records == want["records"]
    assert got.sum_id == want["sum_id"] and got.sum_score_e6 == want["sum_score_e6"]
    assert got.total_e6 == want["total_e6"]
    assert abs(got.total_f64 - want["total_f64"]) <= 1e-12 * max(1.0, abs(want["total_f64"]))


def test_adversarial_1gib_speculative_index(engine):
    import torch

    from falx_gb300 import speculation

    model, _ = speculation.train_model(engine, train_bytes=128 << 20, epochs=2, stride=512)
    host = gen.generate(gen.ADVERSARIAL, 1 << 30)
    data = torch.from_numpy(host.copy()).cuda()
    plain = engine.index_structurals(data, fx.CSV_HASH)
    spec, _, _ = engine.index_structurals_speculative(data, fx.CSV_HASH, model)
    assert torch.equal(plain, spec)
    want = oracle.index_par(host, oracle.CSV_HASH, THREADS)
    assert np.array_equal(plain.cpu().numpy().view(np.uint32), want)
    model.close()


def test_batch_6gib_sample(engine):
    import torch

    from falx_gb300 import batch

    ndocs, total = 4096, 6 << 30
    sizes = batch.mixed_sizes(ndocs, total)
    dialects = batch.mixed_dialects(ndocs)
    host, offs, lens = batch.generate(sizes, dialects)
    data = torch.from_numpy(host).cuda()
    b = batch.Batch(engine, data, offs, lens, dialects)
    b.run()
    rng = np.random.default_rng(20261204)
    sample = sorted(set(rng.choice(ndocs, 48, replace=False).tolist()) | {int(np.argmax(lens))})
    for k in sample:
        doc = host[offs[k]: offs[k] + lens[k]]
        d = int(dialects[k])
        assert b.docs[k].status == 0, k
        idx, c0, v0, c1, v1 = b.result(k)
        assert np.array_equal(idx, oracle.index_par(doc, d, THREADS)), ("index", k, d)
        f0, f1 = batch.GEO_FIELDS[d]
        r = oracle.parse_par(doc, d, [(f0, fx.F64), (f1, fx.F64)], THREADS, index=False, field_bytes=False)
        assert b.docs[k].rows == r["rows"], ("rows", k)
        assert np.array_equal(c0.view(np.uint64), r["columns"][0]["values"].view(np.uint64)), ("col0", k)
        assert np.array_equal(c1.view(np.uint64), r["columns"][1]["values"].view(np.uint64)), ("col1", k)
        assert np.array_equal(v0, r["columns"][0]["valid"]) and np.array_equal(v1, r["columns"][1]["valid"])
    b.close()
