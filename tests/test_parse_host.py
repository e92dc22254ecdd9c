"""Host-buffer entry point (falx_parse_host): input copied in, index and
columns copied back (the index on its own stream while the columns kernel
runs), checked against the oracle."""

import ctypes

import numpy as np
import pytest

import falx_gb300 as fx
import oracle
from falx_gb300 import _lib, gen

pytestmark = pytest.mark.gpu

COLS = [(0, fx.U32), (1, fx.STR), (3, fx.U32), (4, fx.F64), (5, fx.F64)]


def parse_host(engine, doc, dialect, cols):
    n = len(doc)
    src = np.frombuffer(doc, dtype=np.uint8).copy() if n else np.zeros(1, dtype=np.uint8)
    idx_cap, rows_cap, str_cap = n // 2 + 64, n // 2 + 64, n + 64
    index = np.zeros(idx_cap, dtype=np.uint32)
    hcols = _lib.falx_columns()
    hcols.rows_cap = rows_cap
    keep = []
    for k, (_, t) in enumerate(cols):
        if t == fx.STR:
            v = np.zeros(rows_cap + 1, dtype=np.int32)
            sd = np.zeros(str_cap, dtype=np.uint8)
            hcols.cols[k].str_data = sd.ctypes.data
            hcols.cols[k].str_cap = str_cap
        else:
            v = np.zeros(rows_cap, dtype=np.float64 if t == fx.F64 else np.uint32)
            sd = None
        valid = np.zeros((rows_cap + 63) // 64, dtype=np.uint64)
        hcols.cols[k].values = v.ctypes.data
        hcols.cols[k].valid = valid.ctypes.data
        keep.append((v, valid, sd))
    out = _lib.falx_outputs()
    out.index = index.ctypes.data
    out.index_cap = idx_cap
    out.columns = ctypes.pointer(hcols)
    cs = fx.Schema(dialect, cols).to_c()
    _lib.check(engine.lib.falx_parse_host(engine.ctx, ctypes.byref(cs), ctypes.c_void_p(src.ctypes.data), n,
                                          ctypes.byref(out)), "falx_parse_host")
    return index[: out.n_index], hcols.rows, keep, [hcols.cols[k].str_len for k in range(len(cols))]


# 80 MiB and up: the input is copied in chunks and the index kernel starts
# on the first chunk (each tile waits for its own chunk's arrival flag).
@pytest.mark.parametrize("kind,dialect,size", [(gen.CSV_HASH, fx.CSV_HASH, 4 << 20), (gen.ADVERSARIAL, fx.CSV_HASH, 3 << 20),
                                               (gen.CSV_GEO, fx.CSV, 1 << 20), (gen.CSV_HASH, fx.CSV_HASH, 777),
                                               (gen.CSV_HASH, fx.CSV_HASH, 80 << 20),
                                               (gen.ADVERSARIAL, fx.CSV_HASH, (72 << 20) + 12345)])
def test_parse_host_matches_oracle(engine, kind, dialect, size):
    doc = bytes(gen.generate(kind, size))
    for rep in range(2):  # the second call reuses the context's buffers and copy stream
        index, rows, keep, str_len = parse_host(engine, doc, dialect, COLS)
        assert np.array_equal(index, oracle.index_spec(doc, dialect))
        nrows, want = oracle.parse_columns(doc, dialect, COLS)
        assert rows == nrows
        words = (rows + 63) // 64
        for k, (_, t) in enumerate(COLS):
            v, valid, sd = keep[k]
            assert np.array_equal(valid[:words], np.asarray(want[k]["valid"], dtype=np.uint64)), (rep, k)
            if t == fx.STR:
                assert np.array_equal(v[: rows + 1], want[k]["offsets"]), (rep, k)
                assert bytes(sd[: str_len[k]]) == want[k]["data"], (rep, k)
            else:
                assert np.array_equal(v[:rows].view(np.uint8), np.asarray(want[k]["values"]).view(np.uint8)), (rep, k)
