"""Python view of the CPU oracle (oracle.c, oracle_par.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, as the checker or the timed CPU baseline.
The product (falx_gb300) never imports it.

Parity: pinned through the known-answer vectors of the reference's own tests
(tests/golden/), since the reference (a Rust crate) cannot be built here.
"""

import ctypes
from ctypes import POINTER, Structure, byref, c_double, c_int, c_int64, c_uint32, c_uint64, c_void_p

import numpy as np

from . import build as _build

CSV, CSV_HASH, TSV, LOGFMT, NDJSON = 0, 1, 2, 3, 4
I64, U32, F64, STR, BYTES = 0, 1, 2, 3, 4


class orc_col(Structure):
    _fields_ = [("field", c_uint32), ("type", c_uint32), ("values", c_void_p), ("str_data", c_void_p),
                ("str_cap", c_uint64), ("str_len", c_uint64), ("valid", c_void_p)]


class orc_geo_stats(Structure):
    _fields_ = [("records", c_uint64), ("values", c_uint64 * 2), ("checksum", c_uint64 * 2),
                ("sum_e6", c_int64 * 2), ("inexact", c_uint64 * 2), ("fold", c_double * 2)]


class orc_text_stats(Structure):
    _fields_ = [("records", c_uint64), ("city_values", c_uint64), ("city_bytes", c_uint64),
                ("city_checksum", c_uint64), ("values", c_uint64 * 2), ("checksum", c_uint64 * 2)]


class orc_ndjson_stats(Structure):
    _fields_ = [("records", c_uint64), ("sum_id", c_int64), ("sum_score_e6", c_int64), ("total_e6_lo", c_int64),
                ("total_e6_hi", c_int64), ("total_f64", c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        l = ctypes.CDLL(_build.build())
        l.orc_index_spec.restype = c_uint64
        l.orc_index_spec.argtypes = [c_int, c_void_p, c_uint64, c_void_p, c_uint64]
        l.orc_index_seeded.restype = c_uint64
        l.orc_index_seeded.argtypes = [c_int, c_void_p, c_uint64, c_uint32, c_int, c_uint64, c_void_p, c_uint64,
                                       POINTER(c_uint32), POINTER(c_uint64), POINTER(c_uint64)]
        l.orc_index_blocks.restype = c_uint64
        l.orc_index_blocks.argtypes = [c_int, c_void_p, c_uint64, c_void_p, c_uint64]
        l.orc_parse_tape.restype = None
        l.orc_parse_tape.argtypes = [c_int, c_void_p, c_uint64, c_void_p, c_uint64, c_void_p, c_uint64,
                                     POINTER(c_uint64), POINTER(c_uint64)]
        l.orc_parse_columns.restype = c_int
        l.orc_parse_columns.argtypes = [c_int, c_void_p, c_uint64, POINTER(orc_col), c_int, c_uint64,
                                        POINTER(c_uint64)]
        l.orc_geo_stats_run.restype = None
        l.orc_geo_stats_run.argtypes = [c_int, c_void_p, c_uint64, c_uint32, c_uint32, POINTER(orc_geo_stats)]
        l.orc_field_bytes.restype = None
        l.orc_field_bytes.argtypes = [c_int, c_void_p, c_uint64, POINTER(c_uint64), POINTER(c_uint64)]
        l.orc_ndjson_literal.restype = c_int
        l.orc_ndjson_literal.argtypes = [c_void_p, c_uint64, POINTER(c_uint64), POINTER(c_int64)]
        l.orc_ndjson_json.restype = c_int
        l.orc_ndjson_json.argtypes = [c_void_p, c_uint64, POINTER(orc_ndjson_stats)]
        l.orc_parse_f64.restype = c_int
        l.orc_parse_f64.argtypes = [c_void_p, c_uint64, POINTER(c_double)]
        l.orc_parse_i64.restype = c_int
        l.orc_parse_i64.argtypes = [c_void_p, c_uint64, POINTER(c_int64)]
        l.orc_parse_u32.restype = c_int
        l.orc_parse_u32.argtypes = [c_void_p, c_uint64, POINTER(c_uint32)]
        l.orc_par_index.restype = c_uint64
        l.orc_par_index.argtypes = [c_int, c_void_p, c_uint64, c_int, c_void_p, c_uint64]
        l.orc_par_columns.restype = c_int
        l.orc_par_columns.argtypes = [c_int, c_void_p, c_uint64, c_int, POINTER(orc_col), c_int, c_uint64,
                                      POINTER(c_uint64)]
        l.orc_par_parse.restype = c_int
        l.orc_par_parse.argtypes = [c_int, c_void_p, c_uint64, c_int, c_void_p, c_uint64, POINTER(c_uint64),
                                    POINTER(orc_col), c_int, c_uint64, POINTER(c_uint64), POINTER(c_uint64),
                                    POINTER(c_uint64), c_uint32, c_uint32, POINTER(orc_geo_stats)]
        l.orc_par_ndjson_json.restype = c_int
        l.orc_par_ndjson_json.argtypes = [c_void_p, c_uint64, c_int, POINTER(orc_ndjson_stats)]
        l.orc_par_geo_stats.restype = None
        l.orc_par_geo_stats.argtypes = [c_int, c_void_p, c_uint64, c_int, c_uint32, c_uint32, POINTER(orc_geo_stats)]
        l.orc_geo_text_stats.restype = None
        l.orc_geo_text_stats.argtypes = [c_int, c_void_p, c_uint64, c_uint32, c_uint32, c_uint32,
                                         POINTER(orc_text_stats)]
        l.falx_gen.restype = c_uint64
        l.falx_gen.argtypes = [c_int, c_uint64, c_uint64, c_void_p, c_uint64, c_int]
        l.orc_inflate.restype = c_int
        l.orc_inflate.argtypes = [c_void_p, c_uint64, c_void_p, c_uint64]
        l.orc_bgzf_scan.restype = c_int64
        l.orc_bgzf_scan.argtypes = [c_void_p, c_uint64, c_void_p, c_uint64, POINTER(c_uint64)]
        l.orc_bgzf_inflate_par.restype = c_uint64
        l.orc_bgzf_inflate_par.argtypes = [c_void_p, c_void_p, c_uint64, c_void_p, c_void_p, c_int]
        l.orc_par_field_bytes.restype = None
        l.orc_par_field_bytes.argtypes = [c_int, c_void_p, c_uint64, c_int, POINTER(c_uint64), POINTER(c_uint64)]
        _lib = l
    return _lib


def _buf(data):
    a = np.frombuffer(data, dtype=np.uint8) if not isinstance(data, np.ndarray) else np.ascontiguousarray(data)
    return a, a.ctypes.data_as(c_void_p), a.size


def index_spec(data, dialect):
    a, p, n = _buf(data)
    cnt = lib().orc_index_spec(dialect, p, n, None, 0)
    out = np.zeros(max(cnt, 1), dtype=np.uint32)
    lib().orc_index_spec(dialect, p, n, out.ctypes.data_as(c_void_p), cnt)
    return out[:cnt]


NSTATES = {CSV: 2, CSV_HASH: 3, TSV: 1, LOGFMT: 4, NDJSON: 4}


def index_seeded(data, dialect, state=0, prev_byte=-1, pos_base=0):
    """Seeded serial pass over a shard: (index, exit state, terminators, rows)."""
    a, p, n = _buf(data)
    ex, t, r = c_uint32(), c_uint64(), c_uint64()
    cnt = lib().orc_index_seeded(dialect, p, n, state, prev_byte, pos_base, None, 0, byref(ex), byref(t), byref(r))
    out = np.zeros(max(cnt, 1), dtype=np.uint32)
    lib().orc_index_seeded(dialect, p, n, state, prev_byte, pos_base, out.ctypes.data_as(c_void_p), cnt, byref(ex),
                           byref(t), byref(r))
    return out[:cnt], ex.value, t.value, r.value


def shard_summary(data, dialect, prev_byte=-1):
    """Entry-independent summary of a shard: per entry state its exit state
    and its structural / terminator / row counts."""
    out = []
    for s in range(NSTATES[dialect]):
        idx, ex, t, r = index_seeded(data, dialect, s, prev_byte)
        out.append({"exit": ex, "structurals": int(idx.size), "terminators": t, "rows": r})
    return out


def index_blocks(data, dialect):
    a, p, n = _buf(data)
    cnt = lib().orc_index_blocks(dialect, p, n, None, 0)
    out = np.zeros(max(cnt, 1), dtype=np.uint32)
    lib().orc_index_blocks(dialect, p, n, out.ctypes.data_as(c_void_p), cnt)
    return out[:cnt]


def index_par(data, dialect, threads):
    a, p, n = _buf(data)
    cap = n + 1
    out = np.zeros(cap, dtype=np.uint32)
    cnt = lib().orc_par_index(dialect, p, n, threads, out.ctypes.data_as(c_void_p), cap)
    return out[:cnt]


def parse_tape(data, dialect):
    a, p, n = _buf(data)
    ns, ne = c_uint64(), c_uint64()
    lib().orc_parse_tape(dialect, p, n, None, 0, None, 0, byref(ns), byref(ne))
    seps = np.zeros(max(ns.value, 1), dtype=np.uint32)
    ends = np.zeros(max(ne.value, 1), dtype=np.uint64)
    lib().orc_parse_tape(dialect, p, n, seps.ctypes.data_as(c_void_p), ns.value, ends.ctypes.data_as(c_void_p),
                         ne.value, byref(ns), byref(ne))
    return seps[: ns.value], ends[: ne.value]


def _alloc_cols(columns, rows_cap, str_cap):
    cols = (orc_col * max(len(columns), 1))()
    keep = []
    for k, (f, t) in enumerate(columns):
        if t == I64:
            v = np.zeros(max(rows_cap, 1), dtype=np.int64)
        elif t == U32:
            v = np.zeros(max(rows_cap, 1), dtype=np.uint32)
        elif t == F64:
            v = np.zeros(max(rows_cap, 1), dtype=np.float64)
        elif t == BYTES:
            v = np.zeros(max(2 * rows_cap, 1), dtype=np.uint32)
        else:
            v = np.zeros(rows_cap + 1, dtype=np.int32)
        valid = np.zeros(max((rows_cap + 63) // 64, 1), dtype=np.uint64)
        sd = np.zeros(max(str_cap, 1), dtype=np.uint8) if t == STR else None
        cols[k].field = f
        cols[k].type = t
        cols[k].values = v.ctypes.data_as(c_void_p)
        cols[k].valid = valid.ctypes.data_as(c_void_p)
        if sd is not None:
            cols[k].str_data = sd.ctypes.data_as(c_void_p)
            cols[k].str_cap = str_cap
        keep.append((v, valid, sd))
    return cols, keep


def _collect(columns, cols, keep, rows):
    out = []
    words = (rows + 63) // 64
    for k, (f, t) in enumerate(columns):
        v, valid, sd = keep[k]
        c = {"valid": valid[:words].copy()}
        if t == STR:
            c["offsets"] = v[: rows + 1].copy()
            c["data"] = sd[: cols[k].str_len].tobytes()
        elif t == BYTES:
            c["spans"] = v[: 2 * rows].reshape(-1, 2).copy()
        else:
            c["values"] = v[:rows].copy()
        out.append(c)
    return out


def parse_columns(data, dialect, columns, par_threads=0):
    """Columns as a list of dicts (values / valid / offsets / data / spans)."""
    a, p, n = _buf(data)
    rows_cap = n + 1
    str_cap = n + 1
    cols, keep = _alloc_cols(columns, rows_cap, str_cap)
    rows = c_uint64()
    if par_threads:
        rc = lib().orc_par_columns(dialect, p, n, par_threads, cols, len(columns), rows_cap, byref(rows))
    else:
        rc = lib().orc_parse_columns(dialect, p, n, cols, len(columns), rows_cap, byref(rows))
    assert rc == 0
    return rows.value, _collect(columns, cols, keep, rows.value)


def parse_par(data, dialect, columns, threads, index=True, field_bytes=True, stats_fields=None):
    """Index, field bytes, columns and count / sum from one parallel pass
    per chunk: {"index", "field_bytes", "rows", "columns", "stats"}."""
    a, p, n = _buf(data)
    rows_cap = n // 4 + 64
    cols, keep = _alloc_cols(columns, rows_cap, n + 1)
    idx = np.empty(n // 2 + 64, dtype=np.uint32) if index else None
    ni, rows, f, b = c_uint64(), c_uint64(), c_uint64(), c_uint64()
    st = orc_geo_stats() if stats_fields else None
    sf = stats_fields or (0, 0)
    rc = lib().orc_par_parse(dialect, p, n, threads, idx.ctypes.data_as(c_void_p) if index else None,
                             idx.size if index else 0, byref(ni) if index else None, cols, len(columns), rows_cap,
                             byref(rows), byref(f) if field_bytes else None, byref(b) if field_bytes else None,
                             sf[0], sf[1], byref(st) if st is not None else None)
    assert rc == 0
    return {"index": idx[: ni.value] if index else None, "field_bytes": (f.value, b.value) if field_bytes else None,
            "rows": rows.value, "columns": _collect(columns, cols, keep, rows.value), "stats": st}


def geo_stats_par(data, dialect, f0, f1, threads):
    a, p, n = _buf(data)
    st = orc_geo_stats()
    lib().orc_par_geo_stats(dialect, p, n, threads, f0, f1, byref(st))
    return st


def geo_text_stats(data, dialect, city, lat, lon):
    a, p, n = _buf(data)
    st = orc_text_stats()
    lib().orc_geo_text_stats(dialect, p, n, city, lat, lon, byref(st))
    return st


def geo_stats(data, dialect, f0, f1):
    a, p, n = _buf(data)
    st = orc_geo_stats()
    lib().orc_geo_stats_run(dialect, p, n, f0, f1, byref(st))
    return st


def field_bytes(data, dialect, par_threads=0):
    a, p, n = _buf(data)
    f, b = c_uint64(), c_uint64()
    if par_threads:
        lib().orc_par_field_bytes(dialect, p, n, par_threads, byref(f), byref(b))
    else:
        lib().orc_field_bytes(dialect, p, n, byref(f), byref(b))
    return f.value, b.value


def ndjson_literal(data):
    a, p, n = _buf(data)
    r, s = c_uint64(), c_int64()
    rc = lib().orc_ndjson_literal(p, n, byref(r), byref(s))
    return None if rc else (r.value, s.value)


def ndjson_json(data, threads=0):
    a, p, n = _buf(data)
    st = orc_ndjson_stats()
    rc = lib().orc_par_ndjson_json(p, n, threads, byref(st)) if threads else lib().orc_ndjson_json(p, n, byref(st))
    if rc:
        return None
    total = (int(st.total_e6_hi) << 64) | (int(st.total_e6_lo) & ((1 << 64) - 1))
    return {"records": st.records, "sum_id": st.sum_id, "sum_score_e6": st.sum_score_e6, "total_e6": total,
            "total_f64": st.total_f64}


def parse_f64(cell):
    v = c_double()
    a, p, n = _buf(cell)
    return v.value if lib().orc_parse_f64(p, n, byref(v)) else None


def parse_i64(cell):
    v = c_int64()
    a, p, n = _buf(cell)
    return v.value if lib().orc_parse_i64(p, n, byref(v)) else None


def parse_u32(cell):
    v = c_uint32()
    a, p, n = _buf(cell)
    return v.value if lib().orc_parse_u32(p, n, byref(v)) else None


# Seeded synthetic documents (the generator compiled into this library; the
# same bytes as the package's generator for the same kind, size and seed).
GEN_CSV_GEO, GEN_CSV_HASH, GEN_NDJSON, GEN_TSV, GEN_LOGFMT, GEN_ADVERSARIAL = 0, 1, 2, 3, 4, 5
GEN_SEEDS = {0: 0xDEADBEEFCAFEBABE, 1: 0xC0FFEE15600DF00D, 2: 0x853C49E6748FEA9B, 3: 0xA0761D6478BD642F,
             4: 0xE7037ED1A0B428DB, 5: 0x5EEDC5A51234ABCD}


def generate(kind, target_bytes, seed=None, threads=None):
    import os

    seed = GEN_SEEDS[kind] if seed is None else seed
    threads = threads or os.cpu_count() or 1
    buf = np.empty(target_bytes + (1 << 20), dtype=np.uint8)
    n = lib().falx_gen(kind, seed, target_bytes, buf.ctypes.data_as(c_void_p), buf.size, threads)
    if n > buf.size:
        raise ValueError("output buffer too small")
    return buf[:n]


# ---- raw DEFLATE / bgzf (inflate.c)
GZ_BLOCK = np.dtype([("in_off", "<u8"), ("out_off", "<u8"), ("in_len", "<u4"), ("out_len", "<u4")])


def inflate(payload, out_len):
    """(status, bytes) of one raw DEFLATE stream of out_len bytes."""
    a, p, n = _buf(payload)
    out = np.zeros(max(out_len, 1), dtype=np.uint8)
    rc = lib().orc_inflate(p, n, out.ctypes.data_as(c_void_p), out_len)
    return rc, out[:out_len].tobytes()


def bgzf_scan(comp):
    """Structured array of the non-empty members (in_off, out_off, in_len,
    out_len) and the inflated length, or None if malformed."""
    a, p, n = _buf(comp)
    total = c_uint64()
    k = lib().orc_bgzf_scan(p, n, None, 0, byref(total))
    if k < 0:
        return None, 0
    blocks = np.zeros(max(k, 1), dtype=GZ_BLOCK)
    lib().orc_bgzf_scan(p, n, blocks.ctypes.data_as(c_void_p), k, byref(total))
    return blocks[:k], total.value


def bgzf_inflate_par(comp, threads=0):
    """(inflated uint8 array, per-block status) of a bgzf stream."""
    import os

    a, p, n = _buf(comp)
    blocks, total = bgzf_scan(a)
    if blocks is None:
        raise ValueError("not a bgzf stream")
    out = np.empty(max(total, 1), dtype=np.uint8)
    status = np.zeros(max(len(blocks), 1), dtype=np.int32)
    lib().orc_bgzf_inflate_par(p, blocks.ctypes.data_as(c_void_p), len(blocks), out.ctypes.data_as(c_void_p),
                               status.ctypes.data_as(c_void_p), threads or os.cpu_count() or 1)
    return out[:total], status[: len(blocks)]
