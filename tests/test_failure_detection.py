"""Failure detection without a GPU fault: a columns-pass look-back whose
predecessor never publishes gives up after a short bounded wait, the call
returns FALX_ERR_TIMEOUT, and the same context then parses correctly."""

import ctypes
import time

import numpy as np
import pytest

import falx_gb300 as fx
import oracle
from falx_gb300 import _lib, gen

pytestmark = pytest.mark.gpu

COLS = [(0, fx.U32), (1, fx.STR), (4, fx.F64)]


def test_stalled_lookback_times_out_and_context_recovers(engine):
    doc = bytes(gen.generate(gen.CSV_HASH, 256 << 10))  # several thousand records
    d = engine.to_device(doc)
    engine._sync_stream()
    schema = fx.Schema(fx.CSV_HASH, COLS)
    cs = schema.to_c()
    rows_cap, str_cap = len(doc) // 8 + 64, len(doc) + 64
    bufs = engine.alloc_columns(schema, rows_cap, str_cap)
    cols = engine.columns_struct(schema, bufs, rows_cap, str_cap)
    t0 = time.perf_counter()
    rc = engine.lib.falx_test_stalled_lookback(engine.ctx, ctypes.byref(cs), ctypes.c_void_p(d.data_ptr()), d.numel(),
                                               ctypes.byref(cols), 20_000_000)  # 20 ms
    took = time.perf_counter() - t0
    assert rc == _lib.FALX_ERR_TIMEOUT
    assert took < 2.0
    # the context is still usable: a normal call gives the oracle's columns
    got = engine.parse_columns(doc, schema)
    rows, want = oracle.parse_columns(doc, fx.CSV_HASH, COLS)
    assert got.rows == rows
    for k, (_, t) in enumerate(COLS):
        h = got.host(k)
        assert np.array_equal(h["valid"], want[k]["valid"])
        if t == fx.STR:
            assert np.array_equal(h["offsets"], want[k]["offsets"])
            assert h["data"] == want[k]["data"]
        else:
            assert np.array_equal(h["values"].view(np.uint8), np.asarray(want[k]["values"]).view(np.uint8))
