"""Both ways of making rows give the oracle's outputs: the default (index +
tape pass, then the record-parallel pass over the tape) and the fused tile
pass (FALX_OPT_ROWS_PATH = 1)."""

import numpy as np
import pytest

import falx_gb300 as fx
import oracle
from falx_gb300 import _lib, gen
from test_gpu_parity import FUSED_COLS, GEO_COLS, TYPED_COLS, compare_columns, dense_mixed_doc, typed_random_doc
from conftest import Rng

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[0, 1], ids=["tape", "fused"])
def path_engine(request):
    eng = fx.Engine(0)
    assert eng.lib.falx_set_option(eng.ctx, _lib.OPT_ROWS_PATH, request.param) == 0
    yield eng
    eng.close()


@pytest.mark.parametrize("kind,dialect", [(gen.CSV_HASH, fx.CSV_HASH), (gen.ADVERSARIAL, fx.CSV_HASH),
                                          (gen.CSV_GEO, fx.CSV), (gen.TSV, fx.TSV), (gen.LOGFMT, fx.LOGFMT)])
def test_parse_all_paths(path_engine, kind, dialect):
    doc = gen.generate(kind, 3 << 20)
    cols = GEO_COLS if dialect != fx.LOGFMT else [(1, fx.U32), (3, fx.STR), (9, fx.F64), (11, fx.F64)]
    got = path_engine.parse_all(doc, fx.Schema(dialect, cols), stats_fields=(4, 5))
    assert np.array_equal(got["index"].cpu().numpy().view(np.uint32), oracle.index_spec(doc, dialect))
    rows, want = oracle.parse_columns(doc, dialect, cols)
    compare_columns(got["columns"], rows, want, cols)
    fb = got["field_bytes"]
    assert (fb.fields, fb.bytes) == oracle.field_bytes(doc, dialect)
    st, ws = got["stats"], oracle.geo_stats(doc, dialect, 4, 5)
    assert st.records == ws.records and st.values == tuple(ws.values) and st.checksum == tuple(ws.checksum)
    assert st.sum_e6 == tuple(ws.sum_e6) and st.inexact == tuple(ws.inexact)


def test_dense_and_typed_paths(path_engine):
    rng = Rng(0xAB)
    for dialect in (fx.CSV, fx.CSV_HASH, fx.TSV, fx.LOGFMT):
        doc = dense_mixed_doc(rng, dialect, 1 << 20)
        got = path_engine.parse_columns(doc, fx.Schema(dialect, FUSED_COLS))
        rows, want = oracle.parse_columns(doc, dialect, FUSED_COLS)
        compare_columns(got, rows, want, FUSED_COLS)
    docs = b"".join(typed_random_doc(rng) for _ in range(300))
    got = path_engine.parse_columns(docs, fx.Schema(fx.CSV, TYPED_COLS))
    rows, want = oracle.parse_columns(docs, fx.CSV, TYPED_COLS)
    compare_columns(got, rows, want, TYPED_COLS)
    for doc in (b"", b"\n", b"a", b"a\r", b"#x", b"#x\n", b"1,2\n#c\n3,4", b"\n" * 5000, b"," * 70_000):
        for dialect in (fx.CSV, fx.CSV_HASH):
            got = path_engine.parse_columns(doc, fx.Schema(dialect, TYPED_COLS))
            rows, want = oracle.parse_columns(doc, dialect, TYPED_COLS)
            compare_columns(got, rows, want, TYPED_COLS)
