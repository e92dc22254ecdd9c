"""Host-buffer entry point (falx_parse_host): input copied in, index and
columns copied back, checked against the oracle. Inputs of 64 MiB and more
with columns run as a pipeline of input chunks (copies in and out overlap
the parse); the whole-input form (FALX_OPT_PIPELINE 0) must give the same
outputs."""

import ctypes
import random

import numpy as np
import pytest

import falx_gb300 as fx
import oracle
from falx_gb300 import _lib, gen

pytestmark = pytest.mark.gpu

COLS = [(0, fx.U32), (1, fx.STR), (3, fx.U32), (4, fx.F64), (5, fx.F64)]


def parse_host(engine, doc, dialect, cols, tape=False, gz=None):
    """falx_parse_host over `doc`; with gz (a bgzf stream whose text is
    `doc`), falx_parse_gz_host over it instead."""
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
    fb = _lib.falx_field_byte_stats()
    out.field_bytes = ctypes.pointer(fb)
    if tape:
        seps = np.zeros(n + 64, dtype=np.uint32)
        ends = np.zeros(n // 2 + 64, dtype=np.uint64)
        out.seps, out.seps_cap = seps.ctypes.data, seps.size
        out.ends, out.ends_cap = ends.ctypes.data, ends.size
    cs = fx.Schema(dialect, cols).to_c()
    if gz is None:
        _lib.check(engine.lib.falx_parse_host(engine.ctx, ctypes.byref(cs), ctypes.c_void_p(src.ctypes.data), n,
                                              ctypes.byref(out)), "falx_parse_host")
    else:
        from falx_gb300 import bgzf

        blocks, total = bgzf.scan(gz)
        assert total == n
        comp = np.frombuffer(gz, dtype=np.uint8).copy()
        _lib.check(engine.lib.falx_parse_gz_host(engine.ctx, ctypes.byref(cs), ctypes.c_void_p(comp.ctypes.data),
                                                 comp.size, blocks.ctypes.data_as(ctypes.c_void_p), len(blocks),
                                                 ctypes.byref(out)), "falx_parse_gz_host")
    res = (index[: out.n_index], hcols.rows, keep, [hcols.cols[k].str_len for k in range(len(cols))])
    if tape:
        return res + (seps[: out.n_seps], ends[: out.n_ends], (fb.fields, fb.bytes))
    return res


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


def long_records_doc(n_target):
    """Few, long records (about 200 KiB each): chunks of the pipeline that
    hold no whole block of 512 records."""
    rec = b"7," + b"x" * (200 << 10) + b',"a,b",3.5\n'
    return rec * (n_target // len(rec) + 1)


@pytest.mark.parametrize("kind,dialect,size", [(gen.CSV_HASH, fx.CSV_HASH, (100 << 20) + 7),
                                               (gen.CSV_GEO, fx.CSV, 66 << 20),
                                               (gen.ADVERSARIAL, fx.CSV_HASH, 70 << 20),
                                               (None, fx.CSV, 70 << 20)])
def test_pipelined_equals_whole_input(engine, kind, dialect, size):
    doc = bytes(gen.generate(kind, size)) if kind is not None else long_records_doc(size)
    doc = doc[:-1] if doc.endswith(b"\n") else doc  # a trailing record without terminator
    cols = [(0, fx.U32), (1, fx.STR), (2, fx.F64)] if kind is None else COLS
    got = parse_host(engine, doc, dialect, cols, tape=True)
    engine.lib.falx_set_option(engine.ctx, _lib.OPT_PIPELINE, 0)
    try:
        want = parse_host(engine, doc, dialect, cols, tape=True)
    finally:
        engine.lib.falx_set_option(engine.ctx, _lib.OPT_PIPELINE, 1)
    assert np.array_equal(got[0], want[0])
    assert got[1] == want[1]
    assert np.array_equal(got[4], want[4]) and np.array_equal(got[5], want[5]) and got[6] == want[6]
    rows = got[1]
    words = (rows + 63) // 64
    for k, (_, t) in enumerate(cols):
        (v, valid, sd), (w, wvalid, wsd) = got[2][k], want[2][k]
        assert np.array_equal(valid[:words], wvalid[:words]), k
        if t == fx.STR:
            assert got[3][k] == want[3][k]
            assert np.array_equal(v[: rows + 1], w[: rows + 1]) and bytes(sd[: got[3][k]]) == bytes(wsd[: got[3][k]])
        else:
            assert np.array_equal(v[:rows].view(np.uint8), w[:rows].view(np.uint8)), k
    # and the oracle's tape
    s, e = oracle.parse_tape(doc, dialect)
    assert np.array_equal(got[4], s) and np.array_equal(got[5], e)


def same_outputs(got, want, cols):
    assert np.array_equal(got[0], want[0])
    assert got[1] == want[1]
    rows = got[1]
    words = (rows + 63) // 64
    for k, (_, t) in enumerate(cols):
        (v, valid, sd), (w, wvalid, wsd) = got[2][k], want[2][k]
        assert np.array_equal(valid[:words], wvalid[:words]), k
        if t == fx.STR:
            assert got[3][k] == want[3][k]
            assert np.array_equal(v[: rows + 1], w[: rows + 1]) and bytes(sd[: got[3][k]]) == bytes(wsd[: got[3][k]])
        else:
            assert np.array_equal(v[:rows].view(np.uint8), w[:rows].view(np.uint8)), k
    if len(got) > 4:
        assert np.array_equal(got[4], want[4]) and np.array_equal(got[5], want[5]) and got[6] == want[6]


# bgzf text parsed from host buffers (falx_parse_gz_host): the compressed
# bytes copied in, the text inflated in device memory; the same outputs as
# falx_parse_host over the text, in the pipelined form (80 MiB) and the
# whole-input form (3 MiB).
@pytest.mark.parametrize("kind,dialect,size", [(gen.CSV_HASH, fx.CSV_HASH, (80 << 20) + 5),
                                               (gen.ADVERSARIAL, fx.CSV_HASH, 3 << 20),
                                               (gen.CSV_GEO, fx.CSV, 1 << 20)])
def test_parse_gz_host_equals_parse_host(engine, kind, dialect, size):
    from falx_gb300 import bgzf

    doc = bytes(gen.generate(kind, size))
    comp = bgzf.compress(doc, 6)
    want = parse_host(engine, doc, dialect, COLS, tape=True)
    for rep in range(2):  # the second call reuses the compressed-stream buffer and the flags
        got = parse_host(engine, doc, dialect, COLS, tape=True, gz=comp)
        same_outputs(got, want, COLS)


def test_parse_gz_host_errors(engine):
    import ctypes

    from falx_gb300 import bgzf

    doc = bytes(gen.generate(gen.CSV_HASH, 2 << 20))
    comp = bytearray(bgzf.compress(doc, 6))
    blocks, total = bgzf.scan(bytes(comp))
    cs = fx.Schema(fx.CSV_HASH, COLS).to_c()
    out = _lib.falx_outputs()
    buf = np.frombuffer(bytes(comp), dtype=np.uint8).copy()

    def call(b, data):
        return engine.lib.falx_parse_gz_host(engine.ctx, ctypes.byref(cs), ctypes.c_void_p(data.ctypes.data),
                                             data.size, b.ctypes.data_as(ctypes.c_void_p), len(b), ctypes.byref(out))

    # texts not end to end
    bad = blocks.copy()
    bad[3]["out_off"] += 1
    assert call(bad, buf) == _lib.FALX_ERR_INVALID
    # a corrupt member: FALX_ERR_FORMAT
    b = blocks[5]
    comp[int(b["in_off"]) + 3] ^= 0x40
    comp[int(b["in_off"]) + 9] ^= 0x11
    comp[int(b["in_off"]) + 17] ^= 0x08
    broken = np.frombuffer(bytes(comp), dtype=np.uint8).copy()
    status = bgzf.inflate(engine, bytes(comp), blocks, total, status=True)[1]
    assert call(blocks, broken) == (_lib.FALX_ERR_FORMAT if status.any() else _lib.FALX_OK)
    # and the context parses a good stream afterwards
    got = parse_host(engine, doc, fx.CSV_HASH, COLS, gz=bytes(bgzf.compress(doc, 1)))
    assert got[1] == parse_host(engine, doc, fx.CSV_HASH, COLS)[1]
    # an empty stream: no rows
    empty = parse_host(engine, b"", fx.CSV_HASH, COLS, gz=bgzf.EOF_MEMBER)
    assert empty[1] == 0 and len(empty[0]) == 0


def test_parse_gz_host_corrupt_member_at_pipeline_size(engine):
    # a member that fails to inflate in a stream large enough for the
    # pipelined parse: FALX_ERR_FORMAT (the parse ran over whatever the text
    # buffer held), then the same context parses a good stream correctly
    import ctypes

    from falx_gb300 import bgzf

    doc = bytes(gen.generate(gen.CSV_HASH, 72 << 20))
    comp = bytearray(bgzf.compress(doc, 1))
    blocks, total = bgzf.scan(bytes(comp))
    rng = random.Random(5)
    for k in rng.sample(range(len(blocks)), 8):
        b = blocks[k]
        for _ in range(4):
            comp[int(b["in_off"]) + rng.randrange(int(b["in_len"]))] ^= 1 << rng.randrange(8)
    status = bgzf.inflate(engine, bytes(comp), blocks, total, status=True)[1]
    assert status.any()  # (at least one of the damaged members fails)
    cs = fx.Schema(fx.CSV_HASH, COLS).to_c()
    hcols = _lib.falx_columns()
    rows_cap = total // 8
    keep = []
    for k, (_, t) in enumerate(COLS):
        v = np.zeros(rows_cap + 1, dtype=np.float64)  # 8 bytes a row covers every type
        valid = np.zeros((rows_cap + 63) // 64, dtype=np.uint64)
        hcols.cols[k].values = v.ctypes.data
        hcols.cols[k].valid = valid.ctypes.data
        if t == fx.STR:
            sd = np.zeros(total, dtype=np.uint8)
            hcols.cols[k].str_data = sd.ctypes.data
            hcols.cols[k].str_cap = sd.size
            keep.append(sd)
        keep += [v, valid]
    hcols.rows_cap = rows_cap
    out = _lib.falx_outputs()
    out.columns = ctypes.pointer(hcols)
    data = np.frombuffer(bytes(comp), dtype=np.uint8).copy()
    rc = engine.lib.falx_parse_gz_host(engine.ctx, ctypes.byref(cs), ctypes.c_void_p(data.ctypes.data), data.size,
                                       blocks.ctypes.data_as(ctypes.c_void_p), len(blocks), ctypes.byref(out))
    assert rc == _lib.FALX_ERR_FORMAT
    good = bgzf.compress(doc[: 66 << 20], 1)
    got = parse_host(engine, doc[: 66 << 20], fx.CSV_HASH, COLS, gz=good)
    want = parse_host(engine, doc[: 66 << 20], fx.CSV_HASH, COLS)
    same_outputs(got, want, COLS)
