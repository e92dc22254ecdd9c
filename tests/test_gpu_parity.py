"""GPU parity: the CUDA engine (through the C ABI) against the CPU oracle on
seeded inputs, byte-for-byte / bit-for-bit."""

import numpy as np
import pytest

import falx_gb300 as fx
import oracle
from conftest import DIALECT_ALPHABETS, Rng, random_doc
from falx_gb300 import gen

pytestmark = pytest.mark.gpu

DIALECTS = [fx.CSV, fx.CSV_HASH, fx.TSV, fx.LOGFMT, fx.NDJSON]


def gpu_index(engine, doc, dialect):
    return engine.index_structurals(doc, dialect).cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("dialect", DIALECTS)
def test_index_random_small(engine, dialect):
    # Generated-kernel differential inputs (tests/codegen.rs:392-468).
    rng = Rng(0xDEADBEEFCAFEBABE + dialect)
    for _ in range(300):
        doc = random_doc(rng, DIALECT_ALPHABETS[dialect], rng.next() % 300)
        assert np.array_equal(gpu_index(engine, doc, dialect), oracle.index_spec(doc, dialect)), doc


@pytest.mark.parametrize("dialect", DIALECTS)
def test_index_random_long_and_misaligned(engine, dialect):
    # 100 000-byte inputs (tests/codegen.rs:471-543) crossing many tiles,
    # at every base-pointer alignment within 16 bytes.
    rng = Rng(0xCAFEBABEDEADBEEF + dialect)
    doc = random_doc(rng, DIALECT_ALPHABETS[dialect], 100_000)
    big = engine.to_device(doc + b"\0" * 16)
    for off in range(16):
        sub = big[off: off + len(doc) - off]
        want = oracle.index_spec(doc[off:], dialect)
        assert np.array_equal(gpu_index(engine, sub, dialect), want), off


@pytest.mark.parametrize("kind,dialect", [(gen.CSV_GEO, fx.CSV), (gen.CSV_HASH, fx.CSV_HASH), (gen.TSV, fx.TSV),
                                          (gen.LOGFMT, fx.LOGFMT), (gen.NDJSON, fx.NDJSON),
                                          (gen.ADVERSARIAL, fx.CSV_HASH)])
def test_index_generated(engine, kind, dialect):
    doc = gen.generate(kind, 6 << 20)
    assert np.array_equal(gpu_index(engine, doc, dialect), oracle.index_spec(doc, dialect))


@pytest.mark.parametrize("dialect", DIALECTS)
def test_tape(engine, dialect):
    doc = gen.generate({fx.CSV: gen.CSV_GEO, fx.CSV_HASH: gen.ADVERSARIAL, fx.TSV: gen.TSV, fx.LOGFMT: gen.LOGFMT,
                        fx.NDJSON: gen.NDJSON}[dialect], 3 << 20)
    seps, ends = engine.parse_tape(doc, dialect)
    ws, we = oracle.parse_tape(doc, dialect)
    assert np.array_equal(seps.cpu().numpy().view(np.uint32), ws)
    assert np.array_equal(ends.cpu().numpy().view(np.uint64), we)


@pytest.mark.parametrize("doc", [
    b"", b",", b"\n", b"a", b"\r\n", b'"', b'"unterminated,\n,x', b",,,,\n\n\n", b"#", b"#x\n", b'#"\na,b\n',
    b"," * 100_000, b"\n" * 100_000, b'"' * 99_999, b"x" * 70_000,
])
@pytest.mark.parametrize("dialect", DIALECTS)
def test_index_edges(engine, doc, dialect):
    assert np.array_equal(gpu_index(engine, doc, dialect), oracle.index_spec(doc, dialect))


def compare_columns(got, rows, want, cols):
    assert got.rows == rows
    for k, (_, t) in enumerate(cols):
        h = got.host(k)
        assert np.array_equal(h["valid"], want[k]["valid"]), "validity, column %d" % k
        if t == fx.STR:
            assert np.array_equal(h["offsets"], want[k]["offsets"]), "offsets, column %d" % k
            assert h["data"] == want[k]["data"], "arena, column %d" % k
        elif t == fx.BYTES:
            assert np.array_equal(h["spans"], want[k]["spans"]), "spans, column %d" % k
        else:
            assert np.array_equal(h["values"].view(np.uint8), np.asarray(want[k]["values"]).view(np.uint8)), \
                "values, column %d" % k


GEO_COLS = [(0, fx.U32), (1, fx.STR), (2, fx.STR), (3, fx.U32), (4, fx.F64), (5, fx.F64)]
TYPED_COLS = [(0, fx.I64), (1, fx.STR), (2, fx.F64), (4, fx.BYTES)]


@pytest.mark.parametrize("kind,dialect", [(gen.CSV_GEO, fx.CSV), (gen.CSV_HASH, fx.CSV_HASH), (gen.TSV, fx.TSV),
                                          (gen.ADVERSARIAL, fx.CSV_HASH)])
def test_columns_generated(engine, kind, dialect):
    doc = gen.generate(kind, 4 << 20)
    got = engine.parse_columns(doc, fx.Schema(dialect, GEO_COLS))
    rows, want = oracle.parse_columns(doc, dialect, GEO_COLS)
    compare_columns(got, rows, want, GEO_COLS)


def typed_random_doc(rng):
    # The cell mix of tests/columns.rs:454-620 (randomized_differential).
    out = bytearray()
    for _ in range(rng.next() % 40 + 1):
        nf = rng.next() % 8
        crlf = rng.next() % 10 < 1
        for fi in range(nf):
            if fi:
                out += b","
            ct = rng.next() % 7
            if ct == 0:
                sign = b"-" if rng.next() % 2 == 0 else b"+"
                if rng.next() % 3 == 0:
                    out += sign
                out += bytes(48 + rng.next() % 10 for _ in range(rng.next() % 22 + 1))
            elif ct == 1:
                if rng.next() % 2 == 0:
                    out += b"-"
                st = rng.next() % 5
                if st == 0:
                    out += bytes(48 + rng.next() % 10 for _ in range(rng.next() % 18 + 1)) + b"."
                    out += bytes(48 + rng.next() % 10 for _ in range(rng.next() % 18))
                elif st == 1:
                    out += bytes(48 + rng.next() % 10 for _ in range(rng.next() % 15 + 1))
                elif st == 2:
                    out += bytes(48 + rng.next() % 10 for _ in range(rng.next() % 8 + 1)) + b"e"
                    if rng.next() % 2 == 0:
                        out += b"-"
                    e = (rng.next() % (1 << 32)) % 700 - 350
                    out += str(abs(e)).encode()
                elif st == 3:
                    out += b"." + bytes(48 + rng.next() % 10 for _ in range(rng.next() % 15 + 1))
                else:
                    out += bytes(48 + rng.next() % 10 for _ in range(rng.next() % 15 + 1)) + b"."
            elif ct == 2:
                out += bytes(97 + rng.next() % 26 for _ in range(rng.next() % 10))
            elif ct == 3:
                pass
            elif ct == 4:
                out += [b"inf", b"nan", b"NaN"][rng.next() % 3]
            else:
                out += b'"'
                for _ in range(rng.next() % 50):
                    it = rng.next() % 5
                    out += [b",", b'""', b"\n", b" ", bytes([97 + rng.next() % 26])][it]
                out += b'"'
        out += b"\r\n" if crlf else b"\n"
    if rng.next() % 3 == 0:
        for fi in range(rng.next() % 8):
            if fi:
                out += b","
            out += bytes(48 + rng.next() % 10 for _ in range(rng.next() % 20))
    return bytes(out)


def test_columns_typed_random(engine):
    rng = Rng(0xDEADBEEFCAFEBABE)
    docs = [typed_random_doc(rng) for _ in range(200)]
    for doc in docs:
        got = engine.parse_columns(doc, fx.Schema(fx.CSV, TYPED_COLS))
        rows, want = oracle.parse_columns(doc, fx.CSV, TYPED_COLS)
        compare_columns(got, rows, want, TYPED_COLS)
    big = b"".join(docs)
    got = engine.parse_columns(big, fx.Schema(fx.CSV, TYPED_COLS))
    rows, want = oracle.parse_columns(big, fx.CSV, TYPED_COLS)
    compare_columns(got, rows, want, TYPED_COLS)


def test_columns_long_records(engine):
    # Records longer than the halo after a tile: quoted cells of 1-9 KiB.
    rng = Rng(0x1234)
    parts = []
    for i in range(400):
        n = 1000 + rng.next() % 8000 if i % 7 == 0 else rng.next() % 30
        parts.append(b'%d,"%s",x,%d,%d.5,-1.25\n' % (i, b"a,\n#" * (n // 4), i, i))
    doc = b"".join(parts)
    for dialect in (fx.CSV, fx.CSV_HASH):
        got = engine.parse_columns(doc, fx.Schema(dialect, GEO_COLS))
        rows, want = oracle.parse_columns(doc, dialect, GEO_COLS)
        compare_columns(got, rows, want, GEO_COLS)


@pytest.mark.parametrize("doc", [b"", b"\n", b"a", b"a\r", b"\r\n", b"," * 100_000, b"\n" * 100_000,
                                 b'"' * 99_999, b'1,"x\n', b"# c\n#d", b"1,2\n#\n3,4"])
def test_columns_edges(engine, doc):
    for dialect in (fx.CSV, fx.CSV_HASH):
        got = engine.parse_columns(doc, fx.Schema(dialect, TYPED_COLS))
        rows, want = oracle.parse_columns(doc, dialect, TYPED_COLS)
        compare_columns(got, rows, want, TYPED_COLS)


@pytest.mark.parametrize("kind,dialect", [(gen.CSV_HASH, fx.CSV_HASH), (gen.ADVERSARIAL, fx.CSV_HASH),
                                          (gen.CSV_GEO, fx.CSV), (gen.TSV, fx.TSV)])
def test_field_bytes(engine, kind, dialect):
    doc = gen.generate(kind, 4 << 20)
    fb = engine.field_bytes(doc, dialect)
    assert (fb.fields, fb.bytes) == oracle.field_bytes(doc, dialect)


@pytest.mark.parametrize("kind,dialect", [(gen.CSV_GEO, fx.CSV), (gen.CSV_HASH, fx.CSV_HASH)])
def test_geo_stats(engine, kind, dialect):
    doc = gen.generate(kind, 4 << 20)
    st = engine.stats_count_sum(doc, dialect, 4, 5)
    want = oracle.geo_stats(doc, dialect, 4, 5)
    assert st.records == want.records
    assert st.values == tuple(want.values)
    assert st.checksum == tuple(want.checksum)
    assert st.sum_e6 == tuple(want.sum_e6)
    assert st.inexact == tuple(want.inexact)
    for k in range(2):
        # exact fixed point vs the reference's sequential f64 fold
        assert abs(st.sum_f64[k] - want.fold[k]) <= 1e-12 * max(1.0, abs(want.fold[k])) + 1e-9


def test_ndjson_known_answer(engine):
    # tests/ndjson_id_score.rs:5-19: records=3, sum(id + score) = 62.
    doc = (b'{"id":10,"name":"a","tags":["x","y"],"nested":{"score":7,"ok":true},"note":"plain"}\n'
           b'{"id":-3,"name":"quoted \\" id\\":999","tags":["n","m"],"nested":{"score":11,"ok":true},'
           b'"note":"brace } inside"}\n'
           b'{"id":42,"name":"slash \\\\ nested score\\":123","tags":["p","q"],"nested":{"score":-5,"ok":true},'
           b'"note":"end"}\n')
    st = engine.ndjson_id_score(doc)
    assert st.records == 3
    assert st.total_e6 == 62 * 10**6
    assert oracle.ndjson_literal(doc) == (3, 62)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_ndjson_reference_shape_known_answers(engine, seed):
    # known answers from the reference's literal algorithm (ndjson.rs:662-880)
    # on lines of its fixture's shape, many of them across tile boundaries
    from conftest import reference_shape_ndjson

    doc = reference_shape_ndjson(Rng(seed), 60000)
    records, total = oracle.ndjson_literal(doc)
    st = engine.ndjson_id_score(doc)
    assert st.records == records
    assert st.total_e6 == total * 10**6


def test_ndjson_generated(engine):
    doc = gen.generate(gen.NDJSON, 8 << 20)
    st = engine.ndjson_id_score(doc)
    want = oracle.ndjson_json(doc)
    assert st.records == want["records"]
    assert st.sum_id == want["sum_id"]
    assert st.sum_score_e6 == want["sum_score_e6"]
    assert st.total_e6 == want["total_e6"]
    assert st.total_f64 == want["total_f64"]


def ndjson_mixed_doc(rng, size):
    """Stretches of blank and whitespace lines between tiny records (more
    lines per 16 KiB tile than the kernel deals out one per thread), tiny
    records alone, records longer than the 4 KiB staging halo, and
    generated records."""
    out = bytearray()
    stretch = 0
    while len(out) < size:
        kind = stretch % 4
        stretch += 1
        if kind == 0:
            for _ in range(3000):
                k = rng.next() % 4
                out += [b"\n", b" \n", b"\t \n",
                        b'{"id":%d,"nested":{"score":%d}}\n' % (rng.next() % 50, rng.next() % 9)][k]
        elif kind == 1:
            for _ in range(1500):
                out += b'{"id":-%d,"nested":{"score":%d.%d}}\n' % (rng.next() % 999, rng.next() % 99, rng.next() % 9)
        elif kind == 2:
            for _ in range(6):
                pad = b"x" * (3000 + rng.next() % 9000)
                out += b'{"note":"%s","id":%d,"nested":{"ok":true,"score":%d}}\n' % (pad, rng.next() % 7, rng.next() % 5)
        else:
            out += gen.generate(gen.NDJSON, 40_000 + rng.next() % 30_000, seed=rng.next() % 1000).tobytes()
    return bytes(out)


@pytest.mark.parametrize("shift", [0, 5])
def test_ndjson_dense_and_long_lines(engine, shift):
    doc = ndjson_mixed_doc(Rng(77 + shift), 3 << 20)
    buf = engine.to_device(np.frombuffer(b" " * shift + doc, dtype=np.uint8))[shift:]
    st = engine.ndjson_id_score(buf)
    want = oracle.ndjson_json(doc)
    assert want is not None
    assert st.records == want["records"]
    assert st.sum_id == want["sum_id"]
    assert st.sum_score_e6 == want["sum_score_e6"]
    assert st.total_e6 == want["total_e6"]


def dense_mixed_doc(rng, dialect, size):
    """Stretches of very short fields (more structurals per 16 KiB tile than
    the row kernel stages) between stretches of ordinary rows."""
    sep = {fx.CSV: b",", fx.CSV_HASH: b",", fx.TSV: b"\t", fx.LOGFMT: b" "}[dialect]
    out = bytearray()
    while len(out) < size:
        if (len(out) // 40_000) % 2 == 0:
            for _ in range(2000):
                nf = 1 + rng.next() % 6
                cells = []
                for _ in range(nf):
                    k = rng.next() % 6
                    cells.append([b"", b"1", b"-2", b"a", b"3.5", b'""'][k] if dialect != fx.TSV
                                 else [b"", b"1", b"-2", b"a", b"3.5", b"x"][k])
                out += sep.join(cells) + (b"\r\n" if rng.next() % 9 == 0 else b"\n")
                if dialect == fx.CSV_HASH and rng.next() % 17 == 0:
                    out += b"#c,1\n"
        else:
            for _ in range(300):
                out += sep.join([b"%d" % (rng.next() % 100000), b"name%d" % (rng.next() % 97),
                                 b"%d.%06d" % (rng.next() % 90, rng.next() % 10**6),
                                 b"%d" % (rng.next() % 7), b"-%d.25" % (rng.next() % 180), b"%d.5" % (rng.next() % 90)])
                out += b"\n"
    return bytes(out[:size])


FUSED_COLS = [(0, fx.I64), (1, fx.STR), (2, fx.F64), (3, fx.U32), (4, fx.BYTES), (5, fx.STR)]


@pytest.mark.parametrize("dialect", [fx.CSV, fx.CSV_HASH, fx.TSV, fx.LOGFMT])
def test_fused_parse_dense_and_ordinary_tiles(engine, dialect):
    # One falx_parse pass with every output requested, checked output by
    # output against the oracle.
    rng = Rng(0xF00D + dialect)
    doc = dense_mixed_doc(rng, dialect, 3 << 20)
    got = engine.parse_all(doc, fx.Schema(dialect, FUSED_COLS), stats_fields=(2, 5))
    assert np.array_equal(got["index"].cpu().numpy().view(np.uint32), oracle.index_spec(doc, dialect))
    ws, we = oracle.parse_tape(doc, dialect)
    assert np.array_equal(got["seps"].cpu().numpy().view(np.uint32), ws)
    assert np.array_equal(got["ends"].cpu().numpy().view(np.uint64), we)
    rows, want = oracle.parse_columns(doc, dialect, FUSED_COLS)
    compare_columns(got["columns"], rows, want, FUSED_COLS)
    fb = got["field_bytes"]
    assert (fb.fields, fb.bytes) == oracle.field_bytes(doc, dialect)
    st, ws = got["stats"], oracle.geo_stats(doc, dialect, 2, 5)
    assert st.records == ws.records and st.values == tuple(ws.values) and st.checksum == tuple(ws.checksum)
    assert st.sum_e6 == tuple(ws.sum_e6) and st.inexact == tuple(ws.inexact)


@pytest.mark.parametrize("kind,dialect", [(gen.CSV_HASH, fx.CSV_HASH), (gen.ADVERSARIAL, fx.CSV_HASH),
                                          (gen.CSV_GEO, fx.CSV)])
def test_fused_parse_generated(engine, kind, dialect):
    doc = gen.generate(kind, 5 << 20)
    got = engine.parse_all(doc, fx.Schema(dialect, GEO_COLS))
    assert np.array_equal(got["index"].cpu().numpy().view(np.uint32), oracle.index_spec(doc, dialect))
    ws, we = oracle.parse_tape(doc, dialect)
    assert np.array_equal(got["seps"].cpu().numpy().view(np.uint32), ws)
    assert np.array_equal(got["ends"].cpu().numpy().view(np.uint64), we)
    rows, want = oracle.parse_columns(doc, dialect, GEO_COLS)
    compare_columns(got["columns"], rows, want, GEO_COLS)
    fb = got["field_bytes"]
    assert (fb.fields, fb.bytes) == oracle.field_bytes(doc, dialect)


@pytest.mark.parametrize("doc_kind", ["commas", "short_rows"])
def test_dense_inputs_long_lookback(engine, doc_kind):
    # Every tile dense with structurals over tens of MiB: look-back spans of
    # hundreds of tiles sum counts well beyond one tile's 16384.
    doc = b"," * (48 << 20) + b"\n" if doc_kind == "commas" else b"1,2\n" * (24 << 20)
    for dialect in (fx.CSV, fx.CSV_HASH):
        assert np.array_equal(gpu_index(engine, doc, dialect), oracle.index_spec(doc, dialect))
    seps, ends = engine.parse_tape(doc, fx.CSV_HASH)
    ws, we = oracle.parse_tape(doc, fx.CSV_HASH)
    assert np.array_equal(seps.cpu().numpy().view(np.uint32), ws)
    assert np.array_equal(ends.cpu().numpy().view(np.uint64), we)
    if doc_kind == "short_rows":
        cols = [(0, fx.I64), (1, fx.U32)]
        got = engine.parse_columns(doc, fx.Schema(fx.CSV_HASH, cols))
        rows, want = oracle.parse_columns(doc, fx.CSV_HASH, cols)
        compare_columns(got, rows, want, cols)


# Cell shapes around the word-at-a-time decoders' boundaries: digit counts
# 1-10, signs, leading zeros, a non-digit at each position, quoted numbers,
# the d{1,3}.d{6} shape and its near misses, strings of 0-17 bytes.
U32_SHAPES = [b"", b"0", b"7", b"42", b"12345678", b"00000001", b"123456789", b"4294967295", b"4294967296",
              b"99999999999", b"+5", b"-5", b"1a", b"a1", b"1234567a", b"a2345678", b"123 ", b" 123", b'"12"',
              b'"1"2"', b'""', b"1.0", b"\x80", b"9" * 8, b"/", b":"]
F64_SHAPES = [b"0.000000", b"-0.000000", b"+0.000001", b"1.500000", b"-172.432059", b"999.999999", b"1000.000000",
              b"1.5", b"12.3456789", b".123456", b"-.123456", b"1.23456a", b"1a.123456", b"a.123456", b"1.123456e",
              b"+-1.000000", b"1.1234567", b"12.123456", b"123.12345", b"1e5", b"inf", b"NaN", b'"1.500000"',
              b"89.999999", b"-90.000000", b"0.0000005", b"1:.123456", b"1/.123456", b"1,5"]
STR_SHAPES = [b"", b"a", b"ab", b"abc", b"abcd", b"abcde", b"abcdefg", b"abcdefgh", b"abcdefghijklmnopq",
              b'"a""b"', b'""', b'"', b'x"', b'"x', b'"abc"', b"#x", b"\xff\xfe"]
SHAPE_COLS = [(0, fx.U32), (1, fx.I64), (2, fx.F64), (3, fx.STR), (4, fx.U32), (5, fx.F64)]


def shapes_doc(rng, rows):
    out = bytearray()
    for r in range(rows):
        u = U32_SHAPES[r % len(U32_SHAPES)]
        f = F64_SHAPES[(r // 3) % len(F64_SHAPES)]
        s = STR_SHAPES[r % len(STR_SHAPES)]
        u2 = U32_SHAPES[rng.next() % len(U32_SHAPES)]
        f2 = F64_SHAPES[rng.next() % len(F64_SHAPES)]
        out += b",".join([u, u2, f, s, u2, f2])
        out += b"\r\n" if r % 5 == 0 else b"\n"
    return bytes(out)


@pytest.mark.parametrize("dialect", [fx.CSV, fx.CSV_HASH])
def test_columns_cell_shapes(engine, dialect):
    rng = Rng(0x5AA5)
    for rows in (1, 7, 600, 3000):
        doc = shapes_doc(rng, rows)
        got = engine.parse_columns(doc, fx.Schema(dialect, SHAPE_COLS))
        nrows, want = oracle.parse_columns(doc, dialect, SHAPE_COLS)
        compare_columns(got, nrows, want, SHAPE_COLS)
        fb = engine.field_bytes(doc, dialect)
        assert (fb.fields, fb.bytes) == oracle.field_bytes(doc, dialect)
        for f0, f1 in ((2, 5), (0, 3)):
            st = engine.stats_count_sum(doc, dialect, f0, f1)
            want = oracle.geo_stats(doc, dialect, f0, f1)
            assert st.records == want.records
            assert st.values == tuple(want.values)
            assert st.checksum == tuple(want.checksum)
            assert st.sum_e6 == tuple(want.sum_e6)
            assert st.inexact == tuple(want.inexact)
