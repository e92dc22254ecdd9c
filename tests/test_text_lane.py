"""The City text lane (csv_geo_text.rs:1607-1640, sink :1845-1937) on the
GPU against the oracle: records, city values, cleaned bytes and the
wrapping byte checksum, lat / lon values and bit checksums, on generated
csv-geo and csv_hash documents and on hand-made edge rows (quoted cities
with doubled quotes, empty and missing cells, CRLF endings, comments)."""

import pytest

import falx_gb300 as fx
import oracle
from falx_gb300 import gen

pytestmark = pytest.mark.gpu


def check(engine, data, dialect, fields=(1, 4, 5)):
    got = engine.geo_text_stats(data, dialect, fields)
    want = oracle.geo_text_stats(bytes(data), dialect, *fields)
    assert got.records == want.records
    assert (got.city_values, got.city_bytes, got.city_checksum) == \
        (want.city_values, want.city_bytes, want.city_checksum)
    assert (got.latitude_values, got.longitude_values) == tuple(want.values)
    assert (got.latitude_checksum, got.longitude_checksum) == tuple(want.checksum)


@pytest.mark.parametrize("kind,dialect", [(gen.CSV_GEO, fx.CSV), (gen.CSV_HASH, fx.CSV_HASH)])
def test_generated(engine, kind, dialect):
    for size in (1 << 10, 1 << 20, 24 << 20):
        check(engine, gen.generate(kind, size), dialect)


EDGE = (b'id,City,Country,Population,Latitude,Longitude\n'
        b'1,"Ab, C""d""""e",XX,5,1.500000,-2.250000\n'
        b'2,,YY,6,"3.000000",4\n'
        b'3,"",ZZ\n'
        b'4,"x""",AA,7,-90.000000,180.000000\r\n'
        b'5\n'
        b'\n'
        b'6,"' + b'q' * 40 + b'""' + b'r' * 40 + b'",BB,8,0.1,0.2\n'
        b'7,Tail,CC,9,1e3,-0.0')


def test_edge_rows(engine):
    check(engine, EDGE, fx.CSV)
    check(engine, EDGE, fx.CSV, fields=(0, 5, 4))
    hashed = b'# a comment, "with quote\n' + EDGE.replace(b'\n3,', b'\n#3,')
    check(engine, hashed, fx.CSV_HASH)


def test_empty(engine):
    got = engine.geo_text_stats(b"", fx.CSV)
    assert got.records == 0 and got.city_values == 0
