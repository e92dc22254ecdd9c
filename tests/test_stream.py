"""Streaming parser (csv_geo.rs:688-807 StreamParser) on the GPU: documents
fed in chunks of random sizes (single bytes included, chunk edges inside
quoted fields, CRLF pairs, comments and escapes) give the same records, at
the same stream positions and with the same fields, as the whole document
parsed at once by the oracle's tape."""

import numpy as np
import pytest

import falx_gb300 as fx
import oracle
from conftest import DIALECT_ALPHABETS, Rng, random_doc
from falx_gb300 import gen
from falx_gb300.stream import StreamParser

pytestmark = pytest.mark.gpu


def want_records(data, dialect):
    seps, ends = oracle.parse_tape(data, dialect)
    p = fx.Parsed(data, seps, ends, dialect)
    return [((r.start, r.end), r.fields_raw()) for r in p.records()]


def stream_records(engine, data, dialect, cuts):
    sp = StreamParser(dialect, engine)
    got = []
    cb = lambda r: got.append((r.span(), r.fields_raw()))
    prev = 0
    for c in list(cuts) + [len(data)]:
        sp.feed(data[prev:c], cb)
        prev = c
    sp.finish(cb)
    return got


def random_cuts(rng, n, k):
    return sorted({int(rng.next() % (n + 1)) for _ in range(k)})


@pytest.mark.parametrize("kind,dialect", [(gen.CSV_GEO, fx.CSV), (gen.CSV_HASH, fx.CSV_HASH), (gen.TSV, fx.TSV),
                                          (gen.LOGFMT, fx.LOGFMT), (gen.ADVERSARIAL, fx.CSV_HASH)])
def test_generated_in_chunks(engine, kind, dialect):
    data = gen.generate(kind, 300 << 10).tobytes()
    rng = Rng(0x5EED + kind)
    want = want_records(data, dialect)
    assert stream_records(engine, data, dialect, random_cuts(rng, len(data), 40)) == want
    # many small chunks, some a single byte
    cuts = list(range(1, 4000, 7)) + random_cuts(rng, len(data), 20)
    assert stream_records(engine, data, dialect, sorted(set(cuts))) == want


@pytest.mark.parametrize("dialect", [0, 1, 2, 3, 4])
def test_random_alphabet_docs(engine, dialect):
    rng = Rng(0xDEADBEEFCAFEBABE + dialect)
    for _ in range(12):
        doc = random_doc(rng, DIALECT_ALPHABETS[dialect], 1 + rng.next() % 700)
        want = want_records(doc, dialect)
        assert stream_records(engine, doc, dialect, random_cuts(rng, len(doc), 6)) == want


def test_edges(engine):
    doc = b'a,"b\nc",d\r\n# x "y\nq,"""",r\n\n"open\n'
    for dialect in (fx.CSV, fx.CSV_HASH):
        want = want_records(doc, dialect)
        for cut in range(len(doc) + 1):
            assert stream_records(engine, doc, dialect, [cut]) == want, (dialect, cut)
    assert stream_records(engine, b"", fx.CSV, []) == []
    sp = StreamParser(fx.CSV, engine)
    sp.finish(lambda r: None)
    with pytest.raises(RuntimeError):
        sp.feed(b"x", lambda r: None)
