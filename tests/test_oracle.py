"""CPU checks of the oracle: the blockwise restatement of the generated step
kernels against the byte-serial ground truth (the reference's own
differential tests), and the cell decoders against Rust str::parse rules."""

import math
import struct

import numpy as np
import pytest

import oracle
from conftest import DIALECT_ALPHABETS, Rng, random_doc


@pytest.mark.parametrize("dialect", [0, 1, 2, 3, 4])
def test_blocks_match_spec_random(dialect):
    # tests/codegen.rs:392-468: 800 random inputs per format, lengths < 300.
    rng = Rng(0xDEADBEEFCAFEBABE + dialect)
    for _ in range(800):
        doc = random_doc(rng, DIALECT_ALPHABETS[dialect], rng.next() % 300)
        assert np.array_equal(oracle.index_blocks(doc, dialect), oracle.index_spec(doc, dialect)), doc


@pytest.mark.parametrize("dialect", [0, 1, 2, 3, 4])
def test_blocks_match_spec_long(dialect):
    # tests/codegen.rs:471-543: one 100 000-byte input per format.
    rng = Rng(0xCAFEBABEDEADBEEF)
    doc = random_doc(rng, DIALECT_ALPHABETS[dialect], 100_000)
    assert np.array_equal(oracle.index_blocks(doc, dialect), oracle.index_spec(doc, dialect))


def test_interp_matches_scalar_csv():
    # src/lib.rs:48-67: 2000 random CSV inputs over `",\n\rxy`.
    rng = Rng(0xD1B54A32D192ED03)
    for _ in range(2000):
        doc = random_doc(rng, b'",\n\rxy', rng.next() % 300)
        assert np.array_equal(oracle.index_blocks(doc, 0), oracle.index_spec(doc, 0))


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


@pytest.mark.parametrize("cell,expect", [
    (b"1.5", 1.5), (b"-0.0", -0.0), (b"0.1", 0.1), (b"1.5e308", 1.5e308), (b"5e-324", 5e-324),
    (b"inf", math.inf), (b"-inf", -math.inf), (b"Infinity", math.inf), (b".5", 0.5), (b"5.", 5.0),
    (b"+5", 5.0), (b"1e400", math.inf), (b"1e-400", 0.0), (b"-12.345678", -12.345678),
    (b"1_000", None), (b"", None), (b"e5", None), (b"1e", None), (b".", None), (b" 1", None), (b"0x10", None),
    (b"nan(1)", None), (b"+", None), (b"--1", None),
])
def test_parse_f64(cell, expect):
    got = oracle.parse_f64(cell)
    if expect is None:
        assert got is None
    else:
        assert bits(got) == bits(expect)


def test_parse_f64_nan_bits():
    assert bits(oracle.parse_f64(b"NaN")) == 0x7FF8000000000000
    assert bits(oracle.parse_f64(b"-nan")) == 0xFFF8000000000000


@pytest.mark.parametrize("cell,expect", [
    (b"9223372036854775807", 2**63 - 1), (b"-9223372036854775808", -2**63), (b"9223372036854775808", None),
    (b"+5", 5), (b"-0", 0), (b"0007", 7), (b"", None), (b"+", None), (b"-", None), (b"1 ", None), (b"+-1", None),
])
def test_parse_i64(cell, expect):
    assert oracle.parse_i64(cell) == expect


@pytest.mark.parametrize("cell,expect", [
    (b"4294967295", 4294967295), (b"4294967296", None), (b"+7", 7), (b"-0", None), (b"", None), (b"012", 12),
])
def test_parse_u32(cell, expect):
    assert oracle.parse_u32(cell) == expect


@pytest.mark.parametrize("kind,dialect", [(1, 1), (0, 0), (3, 2), (5, 1)])
def test_parallel_port_matches_serial(kind, dialect):
    # The timed CPU baseline (the port of the reference's _par drivers)
    # must agree with the serial restatement at every thread count.
    from falx_gb300 import gen

    doc = gen.generate(kind, 2 << 20)
    cols = [(0, oracle.U32), (1, oracle.STR), (3, oracle.U32), (4, oracle.F64), (5, oracle.F64)]
    serial_rows, serial_cols = oracle.parse_columns(doc, dialect, cols)
    for threads in (1, 2, 3, 7, 16):
        assert np.array_equal(oracle.index_par(doc, dialect, threads), oracle.index_spec(doc, dialect))
        assert oracle.field_bytes(doc, dialect, par_threads=threads) == oracle.field_bytes(doc, dialect)
        rows, got = oracle.parse_columns(doc, dialect, cols, par_threads=threads)
        assert rows == serial_rows
        for k in range(len(cols)):
            for key, v in serial_cols[k].items():
                g = got[k][key]
                if isinstance(v, bytes):
                    assert g == v
                else:
                    assert np.array_equal(np.asarray(g).view(np.uint8), np.asarray(v).view(np.uint8))


def test_ndjson_json_sink_matches_literal_sink_on_reference_shape():
    # the JSON-aware restatement against the reference's literal algorithm
    # (ndjson.rs:662-880, oracle.ndjson_literal) on lines of the reference
    # fixture's shape, where both must accept every line
    from conftest import Rng, reference_shape_ndjson

    for seed in (1, 2, 3):
        doc = reference_shape_ndjson(Rng(seed), 3000)
        lit = oracle.ndjson_literal(doc)
        js = oracle.ndjson_json(doc)
        assert lit is not None and js is not None
        assert js["records"] == lit[0]
        assert js["total_e6"] == lit[1] * 10**6
