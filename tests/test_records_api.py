"""Record and field views over the GPU tape (csv_geo.rs:394-686): the
reference's own record and field answers (tests/comments.rs:13-56), fields
and raw fields of random documents against the oracle's tape, and
parse_into recycling the tape buffers (csv_geo.rs:405)."""

import pytest

import falx_gb300 as fx
import oracle
from conftest import DIALECT_ALPHABETS, Rng, random_doc

pytestmark = pytest.mark.gpu

HAND = (b'# header comment, with "quotes" and, commas\nfoo,42\n#mid, comment\nbar,7\n"#not,a comment",9\n'
        b'# trailing comment')
TRICKY = b'#comment with one " quote\na,"multi\nline"\n#another " stray\nb,2\n'


def test_reference_answers(engine):
    p = fx.parse(HAND, fx.CSV_HASH)
    recs = list(p.records())
    assert [r.as_bytes() for r in recs] == [b"foo,42", b"bar,7", b'"#not,a comment",9']
    # keys are the cleaned first fields, amounts the second (comments.rs:33-40)
    assert [r.fields()[0] for r in recs] == [b"foo", b"bar", b"#not,a comment"]
    assert [int(r.fields()[1]) for r in recs] == [42, 7, 9]
    assert [r.fields_raw()[0] for r in recs] == [b"foo", b"bar", b'"#not,a comment"']
    t = list(fx.parse(TRICKY, fx.CSV_HASH).records())
    assert [r.as_bytes() for r in t] == [b'a,"multi\nline"', b"b,2"]
    assert [r.fields() for r in t] == [[b"a", b"multi\nline"], [b"b", b"2"]]


def split_fields(data, start, end, seps):
    if end > start and data[end - 1] == 0x0D:
        end -= 1
    out, a = [], start
    for s in seps:
        out.append(data[a:int(s)])
        a = int(s) + 1
    out.append(data[a:end])
    return out


@pytest.mark.parametrize("dialect", [0, 1, 2, 3])
def test_fields_match_oracle_tape(engine, dialect):
    rng = Rng(0xC0FFEE + dialect)
    for _ in range(10):
        doc = random_doc(rng, DIALECT_ALPHABETS[dialect], 1 + rng.next() % 900) + b'x\r\n"a""b",c\r\n'
        seps, ends = oracle.parse_tape(doc, dialect)
        want = list(fx.Parsed(doc, seps, ends, dialect).records())
        got = list(fx.parse(doc, dialect).records())
        assert [(r.start, r.end) for r in got] == [(r.start, r.end) for r in want]
        for g, w in zip(got, want):
            raw = split_fields(doc, w.start, w.end, w.seps)
            assert g.fields_raw() == raw
            assert g.fields() == [fx.clean(x) for x in raw]
            assert g.field_count() == len(raw)


def test_parse_into_recycles(engine):
    docs = [b"a,b\nc,d\n" * 40, b'x,"y\nz",w\n1,2\n3\n', b"", b"only"]
    prev = None
    bufs = None
    for d in docs:
        p = fx.parse_into(d, prev, fx.CSV)
        want = [r.fields() for r in fx.parse(d, fx.CSV).records()]
        assert [r.fields() for r in p.records()] == want
        if bufs is not None:
            # the recycled device buffers hold the smaller tapes
            assert p._device[0].data_ptr() == bufs[0].data_ptr()
            assert p._device[1].data_ptr() == bufs[1].data_ptr()
        bufs = p._device
        prev = p
