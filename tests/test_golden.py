"""The oracle (CPU) and the engine (GPU) against the known-answer vectors of
the reference's tests, committed in tests/golden/reference_vectors.json by
tests/golden/make_golden.py."""

import base64
import json
import os
import struct

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "reference_vectors.json")))["cases"]
TYPES = {"i64": oracle.I64, "f64": oracle.F64, "str": oracle.STR, "bytes": oracle.BYTES, "u32": oracle.U32}


def data_of(c):
    return base64.b64decode(c["data"])


def rows_from_columns(schema, rows, cols):
    out = []
    for r in range(rows):
        row = []
        for k, (f, t) in enumerate(schema):
            valid = (int(cols[k]["valid"][r >> 6]) >> (r & 63)) & 1
            if t == "str":
                o = cols[k]["offsets"]
                row.append(base64.b64encode(bytes(cols[k]["data"][int(o[r]):int(o[r + 1])])).decode()
                           if valid else None)
            elif not valid:
                row.append(None)
            elif t == "i64":
                row.append(int(cols[k]["values"][r]))
            elif t == "f64":
                row.append(struct.unpack("<Q", struct.pack("<d", float(cols[k]["values"][r])))[0])
            else:
                row.append([int(x) for x in cols[k]["spans"][r]])
        out.append(row)
    return out


def expected_rows(c):
    return c["columns"]["rows"]


@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference_vectors(c):
    d = data_of(c)
    assert list(oracle.index_spec(d, c["dialect"])) == c["index"]
    assert list(oracle.index_blocks(d, c["dialect"])) == c["index"]
    seps, ends = oracle.parse_tape(d, c["dialect"])
    assert list(seps) == c["seps"] and [int(x) for x in ends] == c["ends"]
    if c.get("field_bytes"):
        assert list(oracle.field_bytes(d, c["dialect"])) == c["field_bytes"]
    if c.get("columns"):
        schema = c["columns"]["schema"]
        rows, cols = oracle.parse_columns(d, c["dialect"], [(f, TYPES[t]) for f, t in schema])
        assert rows_from_columns(schema, rows, cols) == expected_rows(c)
    if c.get("ndjson"):
        assert oracle.ndjson_literal(d) == (c["ndjson"]["records"], c["ndjson"]["sum"])
        assert oracle.ndjson_json(d)["total_e6"] == c["ndjson"]["sum"] * 10**6


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_engine_matches_reference_vectors(engine, c):
    import falx_gb300 as fx

    d = data_of(c)
    idx = engine.index_structurals(d, c["dialect"]).cpu().numpy().view(np.uint32)
    assert list(idx) == c["index"]
    seps, ends = engine.parse_tape(d, c["dialect"])
    hs, he = seps.cpu().numpy().view(np.uint32), ends.cpu().numpy().view(np.uint64)
    assert list(hs) == c["seps"]
    assert [int(x) for x in he] == c["ends"]
    if c.get("records"):
        recs = [r.as_bytes() for r in fx.Parsed(d, hs, he, c["dialect"]).records()]
        assert recs == [base64.b64decode(x) for x in c["records"]]
    if c.get("field_bytes"):
        fb = engine.field_bytes(d, c["dialect"])
        assert [fb.fields, fb.bytes] == c["field_bytes"]
    if c.get("columns"):
        schema = c["columns"]["schema"]
        got = engine.parse_columns(d, fx.Schema(c["dialect"], [(f, TYPES[t]) for f, t in schema]))
        cols = [got.host(k) for k in range(len(schema))]
        assert rows_from_columns(schema, got.rows, cols) == expected_rows(c)
    if c.get("ndjson"):
        st = engine.ndjson_id_score(d)
        assert st.records == c["ndjson"]["records"] and st.total_e6 == c["ndjson"]["sum"] * 10**6
