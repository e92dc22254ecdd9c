"""falx_gb300: GB300 engine for the falx structural-index and
column-materialisation path.

The module mirrors the API of a generated falx parser module (Mapika/falx
src/kernels/csv_geo.rs, csv_hash.rs, csv_typed.rs, tsv.rs, logfmt.rs,
ndjson.rs) with the dialect as an argument:

    index_structurals(data, dialect)           csv_geo.rs:24    (and _par, :95)
    parse(data, dialect) -> Parsed             csv_geo.rs:394   (and parse_par, :215; parse_into, :405)
        Parsed.records() -> Record.fields()    csv_geo.rs:424-686
    parse_columns(data, schema) -> Columns     csv_geo.rs:1112  (and _par :1216, _chunks_par :1167)
    parse_csv_geo_stats(data, ...)             csv_geo.rs:1505  (and _par, :1513)
    parse_csv_geo_text_stats(data, ...)        csv_geo_text.rs:1627  (and _par, :1637)
    parse_field_bytes(data, dialect)           csv_hash.rs:976  (and _par, :984)
    parse_ndjson_id_score(data)                ndjson.rs:679    (and _par, :726)
    bitmap_get, string_at                      csv_geo.rs:1105, csv_hash.rs:1444

`data` is bytes / a NumPy uint8 array (copied to the GPU), or a CUDA uint8
torch tensor (used in place). All work runs in the CUDA engine through the C
ABI in include/falx_gpu.h; `threads` arguments of the `_par` forms are
accepted for drop-in compatibility and ignored (the whole GPU runs every
call). Errors raise FalxError where the reference panics or grows a Vec.
"""

import ctypes
import warnings
from ctypes import byref, c_uint64, c_void_p

import numpy as np

from . import _lib
from ._lib import BYTES, CSV, CSV_HASH, F64, I64, LOGFMT, NDJSON, STR, TSV, U32, FalxError, check

__all__ = [
    "CSV", "CSV_HASH", "TSV", "LOGFMT", "NDJSON", "I64", "U32", "F64", "STR", "BYTES", "FalxError",
    "Engine", "Schema", "Columns", "Parsed", "Record", "index_structurals", "index_structurals_par", "parse",
    "parse_par", "parse_into", "parse_columns", "parse_columns_par", "parse_columns_chunks_par", "parse_csv_geo_stats",
    "parse_csv_geo_stats_par", "parse_csv_geo_text_stats", "parse_csv_geo_text_stats_par", "parse_field_bytes", "parse_field_bytes_par", "parse_ndjson_id_score",
    "parse_ndjson_id_score_par", "bitmap_get", "string_at", "engine",
]


class Schema:
    """A dialect plus projected columns: [(field ordinal, type), ...]
    (codegen.rs:99-110 Column; at most 32 columns)."""

    def __init__(self, dialect, columns=()):
        self.dialect = dialect
        self.columns = list(columns)
        if len(self.columns) > _lib.MAX_COLUMNS:
            raise ValueError("at most %d columns" % _lib.MAX_COLUMNS)

    def to_c(self):
        s = _lib.falx_schema()
        s.dialect = self.dialect
        s.ncols = len(self.columns)
        for k, (f, t) in enumerate(self.columns):
            s.cols[k].field = f
            s.cols[k].type = t
        return s


def _torch():
    import torch

    return torch


class Engine:
    """One engine context on one GPU (falx_create). Not thread-safe."""

    def __init__(self, device=0):
        torch = _torch()
        self.lib = _lib.load()
        self.device = device
        self.torch = torch
        ctx = c_void_p()
        with torch.cuda.device(device):
            torch.cuda.init()
            check(self.lib.falx_create(device, byref(ctx)), "falx_create")
        self.ctx = ctx

    def close(self):
        if self.ctx:
            self.lib.falx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- helpers ---------------------------------------------------------------
    def _sync_stream(self):
        s = self.torch.cuda.current_stream(self.device)
        self.lib.falx_set_stream(self.ctx, c_void_p(s.cuda_stream))

    def to_device(self, data):
        """Device uint8 tensor for `data` (bytes, NumPy, or a tensor)."""
        torch = self.torch
        if isinstance(data, torch.Tensor):
            t = data if data.is_cuda else data.to("cuda:%d" % self.device)
            if t.dtype != torch.uint8 or not t.is_contiguous():
                raise ValueError("data tensor must be contiguous uint8")
            return t
        arr = np.frombuffer(memoryview(data), dtype=np.uint8) if not isinstance(data, np.ndarray) else data
        with warnings.catch_warnings():
            # a read-only view of bytes: torch only reads it, for the copy to the device
            warnings.simplefilter("ignore", UserWarning)
            return torch.from_numpy(np.ascontiguousarray(arr, dtype=np.uint8)).to("cuda:%d" % self.device)

    def empty(self, n, dtype):
        return self.torch.empty(max(int(n), 1), dtype=dtype, device="cuda:%d" % self.device)

    # -- entry points ----------------------------------------------------------
    def index_structurals(self, data, dialect=CSV, cap=None):
        """Structural offsets as an int32 CUDA tensor (values are u32)."""
        d = self.to_device(data)
        n = d.numel()
        self._sync_stream()
        cap = n // 4 + 1024 if cap is None else cap
        while True:
            out = self.empty(cap, self.torch.int32)
            cnt = c_uint64()
            rc = self.lib.falx_index_structurals(self.ctx, dialect, c_void_p(d.data_ptr()), n,
                                                 c_void_p(out.data_ptr()), cap, byref(cnt))
            if rc == _lib.FALX_ERR_CAPACITY and cnt.value > cap:
                cap = cnt.value
                continue
            check(rc, "falx_index_structurals")
            return out[: cnt.value]

    def parse_tape(self, data, dialect=CSV, reuse=None):
        """(seps int32 tensor, ends int64 tensor) of the record tape. `reuse`:
        (seps, ends) device tensors of an earlier tape to write into when
        they are large enough."""
        d = self.to_device(data)
        n = d.numel()
        self._sync_stream()
        if reuse is not None:
            # the recycled buffers first; larger ones only if the tape needs them
            seps, ends = reuse
            scap, ecap = seps.numel(), ends.numel()
        else:
            scap, ecap = n // 4 + 1024, n // 16 + 1024
            seps, ends = None, None
        while True:
            if seps is None:
                seps = self.empty(scap, self.torch.int32)
                ends = self.empty(ecap, self.torch.int64)
            ns, ne = c_uint64(), c_uint64()
            rc = self.lib.falx_parse_tape(self.ctx, dialect, c_void_p(d.data_ptr()), n, c_void_p(seps.data_ptr()),
                                          scap, c_void_p(ends.data_ptr()), ecap, byref(ns), byref(ne))
            if rc == _lib.FALX_ERR_CAPACITY:
                scap, ecap = max(scap, ns.value), max(ecap, ne.value)
                seps = None
                continue
            check(rc, "falx_parse_tape")
            return seps[: ns.value], ends[: ne.value]

    def alloc_columns(self, schema, rows_cap, str_cap):
        """Device buffers for `schema` sized for rows_cap rows."""
        torch = self.torch
        bufs = []
        for f, t in schema.columns:
            if t in (I64,):
                v = self.empty(rows_cap, torch.int64)
            elif t == F64:
                v = self.empty(rows_cap, torch.float64)
            elif t == U32:
                v = self.empty(rows_cap, torch.int32)
            elif t == BYTES:
                v = self.empty(2 * rows_cap, torch.int32)
            else:
                v = self.empty(rows_cap + 1, torch.int32)
            valid = self.empty((rows_cap + 63) // 64, torch.int64)
            sd = self.empty(str_cap, torch.uint8) if t == STR else None
            bufs.append((v, valid, sd))
        return bufs

    def columns_struct(self, schema, bufs, rows_cap, str_cap):
        cols = _lib.falx_columns()
        cols.rows_cap = rows_cap
        for k, (v, valid, sd) in enumerate(bufs):
            cols.cols[k].values = v.data_ptr()
            cols.cols[k].valid = valid.data_ptr()
            if sd is not None:
                cols.cols[k].str_data = sd.data_ptr()
                cols.cols[k].str_cap = str_cap
        return cols

    def parse_columns(self, data, schema, rows_cap=None, str_cap=None):
        d = self.to_device(data)
        n = d.numel()
        self._sync_stream()
        rows_cap = n // 8 + 64 if rows_cap is None else rows_cap
        str_cap = n + 64 if str_cap is None else str_cap
        cs = schema.to_c()
        while True:
            bufs = self.alloc_columns(schema, rows_cap, str_cap)
            cols = self.columns_struct(schema, bufs, rows_cap, str_cap)
            rc = self.lib.falx_parse_columns(self.ctx, byref(cs), c_void_p(d.data_ptr()), n, byref(cols))
            if rc == _lib.FALX_ERR_CAPACITY:
                rows_cap = max(rows_cap, cols.rows)
                str_cap = max([str_cap] + [cols.cols[k].str_len for k in range(len(schema.columns))])
                continue
            check(rc, "falx_parse_columns")
            return Columns(schema, cols.rows, bufs, [cols.cols[k].str_len for k in range(len(schema.columns))], d)

    def parse_all(self, data, schema, stats_fields=(4, 5)):
        """Every output of one fused falx_parse pass: structural index, tape,
        columns, field-byte counts and count/sum stats (stats_fields=None
        leaves the stats out)."""
        torch = self.torch
        d = self.to_device(data)
        n = d.numel()
        self._sync_stream()
        cs = schema.to_c()
        icap, scap, ecap = n // 4 + 64, n // 4 + 64, n // 8 + 64
        rows_cap, str_cap = n // 8 + 64, n + 64
        while True:
            index = self.empty(icap, torch.int32)
            seps = self.empty(scap, torch.int32)
            ends = self.empty(ecap, torch.int64)
            bufs = self.alloc_columns(schema, rows_cap, str_cap)
            cols = self.columns_struct(schema, bufs, rows_cap, str_cap)
            fb = _lib.falx_field_byte_stats()
            st = _lib.falx_geo_stats()
            out = _lib.falx_outputs()
            out.index, out.index_cap = index.data_ptr(), icap
            out.seps, out.seps_cap = seps.data_ptr(), scap
            out.ends, out.ends_cap = ends.data_ptr(), ecap
            out.columns = ctypes.pointer(cols)
            out.field_bytes = ctypes.pointer(fb)
            if stats_fields is not None:
                out.stats = ctypes.pointer(st)
                out.stats_fields[0], out.stats_fields[1] = stats_fields
            rc = self.lib.falx_parse(self.ctx, byref(cs), c_void_p(d.data_ptr()), n, byref(out))
            if rc == _lib.FALX_ERR_CAPACITY:
                icap, scap, ecap = max(icap, out.n_index), max(scap, out.n_seps), max(ecap, out.n_ends)
                rows_cap = max(rows_cap, cols.rows)
                str_cap = max([str_cap] + [cols.cols[k].str_len for k in range(len(schema.columns))])
                continue
            check(rc, "falx_parse")
            columns = Columns(schema, cols.rows, bufs, [cols.cols[k].str_len for k in range(len(schema.columns))], d)
            return {"index": index[: out.n_index], "seps": seps[: out.n_seps], "ends": ends[: out.n_ends],
                    "columns": columns, "field_bytes": FieldByteStats(fb.fields, fb.bytes),
                    "stats": GeoStats(st) if stats_fields is not None else None}

    # ---- learned speculation -------------------------------------------
    def model_create(self, seed=1):
        """A freshly initialised entry-region predictor on this engine's GPU."""
        return EntryModel(self, seed)

    def region_states(self, data, dialect):
        """Exact region state at the start of every 64-byte block (labels)."""
        torch = self.torch
        d = self.to_device(data)
        self._sync_stream()
        n = c_uint64()
        self.lib.falx_region_states(self.ctx, dialect, c_void_p(d.data_ptr()), d.numel(), None, 0, byref(n))
        out = self.empty(max(n.value, 1), torch.uint8)
        check(self.lib.falx_region_states(self.ctx, dialect, c_void_p(d.data_ptr()), d.numel(),
                                          c_void_p(out.data_ptr()), n.value, byref(n)), "falx_region_states")
        return out[: n.value]

    def byte_classes(self, data, starts):
        """Classes of the 256 bytes from each start offset: uint8 [n, 256]."""
        torch = self.torch
        d = self.to_device(data)
        st = starts.to(device=d.device, dtype=torch.int64).contiguous()
        self._sync_stream()
        n = st.numel()
        cls = self.empty(max(n, 1) * _lib.MLP_BYTES, torch.uint8)
        check(self.lib.falx_byte_classes(self.ctx, c_void_p(d.data_ptr()), d.numel(), c_void_p(st.data_ptr()), n,
                                         c_void_p(cls.data_ptr())), "falx_byte_classes")
        return cls[: n * _lib.MLP_BYTES].view(n, _lib.MLP_BYTES)

    def index_structurals_speculative(self, data, dialect, model=None, assumed=None):
        """Speculative structural index: (index, tiles, mispredicted). Entry
        states come from `model`, from the per-tile array `assumed`, or (both
        None) are taken as the file's initial state."""
        torch = self.torch
        d = self.to_device(data)
        self._sync_stream()
        n = d.numel()
        cap = n // 4 + 64
        st = _lib.falx_spec_stats()
        while True:
            out = self.empty(cap, torch.int32)
            cnt = c_uint64()
            if assumed is not None:
                a = assumed.to(device=d.device, dtype=torch.uint8).contiguous()
                rc = self.lib.falx_index_structurals_assumed(self.ctx, dialect, c_void_p(d.data_ptr()), n,
                                                             c_void_p(a.data_ptr()), c_void_p(out.data_ptr()), cap,
                                                             byref(cnt), byref(st))
            else:
                rc = self.lib.falx_index_structurals_speculative(self.ctx, model.ptr if model else None, dialect,
                                                                 c_void_p(d.data_ptr()), n, c_void_p(out.data_ptr()),
                                                                 cap, byref(cnt), byref(st))
            if rc == _lib.FALX_ERR_CAPACITY and cnt.value > cap:
                cap = cnt.value
                continue
            check(rc, "falx_index_structurals_speculative")
            return out[: cnt.value], st.tiles, st.mispredicted

    def stats_count_sum(self, data, dialect, field0, field1):
        d = self.to_device(data)
        self._sync_stream()
        st = _lib.falx_geo_stats()
        check(self.lib.falx_stats_count_sum(self.ctx, dialect, c_void_p(d.data_ptr()), d.numel(), field0, field1,
                                            byref(st)), "falx_stats_count_sum")
        return GeoStats(st)

    def geo_text_stats(self, data, dialect=CSV, fields=(1, 4, 5)):
        """City text lane plus lat / lon counts and checksums
        (csv_geo_text.rs:1627 parse_csv_geo_text_stats); fields = (city,
        latitude, longitude) ordinals."""
        d = self.to_device(data)
        self._sync_stream()
        st = _lib.falx_geo_text_stats()
        check(self.lib.falx_csv_geo_text_stats(self.ctx, dialect, c_void_p(d.data_ptr()), d.numel(), fields[0],
                                               fields[1], fields[2], byref(st)), "falx_csv_geo_text_stats")
        return st

    def field_bytes(self, data, dialect):
        d = self.to_device(data)
        self._sync_stream()
        fb = _lib.falx_field_byte_stats()
        check(self.lib.falx_field_bytes(self.ctx, dialect, c_void_p(d.data_ptr()), d.numel(), byref(fb)),
              "falx_field_bytes")
        return FieldByteStats(fb.fields, fb.bytes)

    def ndjson_id_score(self, data):
        d = self.to_device(data)
        self._sync_stream()
        st = _lib.falx_ndjson_stats()
        check(self.lib.falx_ndjson_id_score(self.ctx, c_void_p(d.data_ptr()), d.numel(), byref(st)),
              "falx_ndjson_id_score")
        return NdjsonIdScoreStats(st)


class EntryModel:
    """Entry-region predictor (falx_model): 256 leading bytes of a tile ->
    NORMAL / QUOTE / COMMENT. Trained and run by the engine's own kernels."""

    def __init__(self, engine, seed=1):
        self.engine = engine
        p = c_void_p()
        check(engine.lib.falx_model_create(engine.ctx, seed, byref(p)), "falx_model_create")
        self.ptr = p

    def close(self):
        if self.ptr:
            self.engine.lib.falx_model_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_confidence(self, min_prob):
        """Tiles predicted with probability below min_prob assume nothing."""
        check(self.engine.lib.falx_model_set_confidence(self.ptr, min_prob), "falx_model_set_confidence")

    @staticmethod
    def param_count():
        return int(_lib.load().falx_model_param_count())

    def get(self):
        w = np.empty(self.param_count(), dtype=np.float32)
        check(self.engine.lib.falx_model_get(self.engine.ctx, self.ptr, c_void_p(w.ctypes.data), w.size),
              "falx_model_get")
        return w

    def set(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        check(self.engine.lib.falx_model_set(self.engine.ctx, self.ptr, c_void_p(w.ctypes.data), w.size),
              "falx_model_set")

    def forward(self, cls):
        """Logits [n, 3] (float32) and the predicted states [n] (uint8)."""
        torch = self.engine.torch
        cls = cls.contiguous()
        n = cls.shape[0]
        z = self.engine.empty(max(n, 1) * 3, torch.float32)
        pred = self.engine.empty(max(n, 1), torch.uint8)
        check(self.engine.lib.falx_model_forward(self.engine.ctx, self.ptr, c_void_p(cls.data_ptr()), n,
                                                 c_void_p(z.data_ptr()), c_void_p(pred.data_ptr())),
              "falx_model_forward")
        return z[: n * 3].view(n, 3), pred[:n]

    def grad(self, cls, labels):
        """Gradient of the mean cross-entropy (flat float32, parameter order
        of falx_model_get) and the loss."""
        torch = self.engine.torch
        g = self.engine.empty(self.param_count(), torch.float32)
        loss = ctypes.c_float()
        check(self.engine.lib.falx_model_grad(self.engine.ctx, self.ptr, c_void_p(cls.contiguous().data_ptr()),
                                              c_void_p(labels.contiguous().data_ptr()), cls.shape[0],
                                              c_void_p(g.data_ptr()), byref(loss)), "falx_model_grad")
        return g, loss.value

    def train(self, cls, labels, batch=512, epochs=1, lr=1e-3):
        loss = ctypes.c_float()
        check(self.engine.lib.falx_model_train(self.engine.ctx, self.ptr, c_void_p(cls.contiguous().data_ptr()),
                                               c_void_p(labels.contiguous().data_ptr()), cls.shape[0], batch, epochs,
                                               lr, byref(loss)), "falx_model_train")
        return loss.value

    def predict_tiles(self, data):
        torch = self.engine.torch
        d = self.engine.to_device(data)
        self.engine._sync_stream()
        tiles = (d.numel() + (d.data_ptr() & 15) + _lib.SPEC_TILE - 1) // _lib.SPEC_TILE
        out = self.engine.empty(max(tiles, 1), torch.uint8)
        n = c_uint64()
        check(self.engine.lib.falx_predict_tiles(self.engine.ctx, self.ptr, c_void_p(d.data_ptr()), d.numel(),
                                                 c_void_p(out.data_ptr()), tiles, byref(n)), "falx_predict_tiles")
        return out[: n.value]


class GeoStats:
    """parse_csv_geo_stats result: the reference's counts and bit checksums
    (csv_geo.rs:1491-1497) plus exact fixed-point sums."""

    def __init__(self, st):
        self.records = st.records
        self.values = tuple(st.values)
        self.checksum = tuple(st.checksum)
        self.sum_e6 = tuple(st.sum_e6)
        self.inexact = tuple(st.inexact)
        self.sum_f64 = tuple(st.sum_f64)

    def __repr__(self):
        return "GeoStats(records=%d, values=%s, checksum=%s, sum_e6=%s)" % (
            self.records, self.values, [hex(c) for c in self.checksum], self.sum_e6)


class FieldByteStats:
    def __init__(self, fields, bytes_):
        self.fields = fields
        self.bytes = bytes_

    def __eq__(self, o):
        return (self.fields, self.bytes) == (o.fields, o.bytes)

    def __repr__(self):
        return "FieldByteStats(fields=%d, bytes=%d)" % (self.fields, self.bytes)


class NdjsonIdScoreStats:
    def __init__(self, st):
        self.records = st.records
        self.sum_id = st.sum_id
        self.sum_score_e6 = st.sum_score_e6
        self.total_e6 = (int(st.total_e6_hi) << 64) | (int(st.total_e6_lo) & ((1 << 64) - 1))
        self.total_f64 = st.total_f64

    def __repr__(self):
        return "NdjsonIdScoreStats(records=%d, total_e6=%d)" % (self.records, self.total_e6)


class Columns:
    """Typed columns (Arrow layout, csv_geo.rs:920-946): per column a values
    tensor and an LSB-first validity bitmap; STR columns have i32 offsets
    (rows + 1) and a byte arena. Tensors live on the GPU; `host()` copies."""

    def __init__(self, schema, rows, bufs, str_lens, data):
        self.schema = schema
        self.rows = rows
        self._bufs = bufs
        self._str_lens = str_lens
        self.data = data

    def column(self, k):
        v, valid, sd = self._bufs[k]
        t = self.schema.columns[k][1]
        words = (self.rows + 63) // 64
        if t == STR:
            return {"offsets": v[: self.rows + 1], "data": sd[: self._str_lens[k]], "valid": valid[:words]}
        if t == BYTES:
            return {"spans": v[: 2 * self.rows].view(-1, 2), "valid": valid[:words]}
        return {"values": v[: self.rows], "valid": valid[:words]}

    def host(self, k):
        """Column k as NumPy arrays with the reference's element types."""
        c = self.column(k)
        t = self.schema.columns[k][1]
        out = {"valid": c["valid"].cpu().numpy().view(np.uint64)}
        if t == STR:
            out["offsets"] = c["offsets"].cpu().numpy()
            out["data"] = c["data"].cpu().numpy().tobytes()
        elif t == BYTES:
            out["spans"] = c["spans"].cpu().numpy().view(np.uint32)
        elif t == U32:
            out["values"] = c["values"].cpu().numpy().view(np.uint32)
        else:
            out["values"] = c["values"].cpu().numpy()
        return out


class Record:
    """One record: a span plus its separator offsets (csv_geo.rs:518-600)."""

    __slots__ = ("data", "start", "end", "seps")

    def __init__(self, data, start, end, seps):
        self.data, self.start, self.end, self.seps = data, start, end, seps

    def _trimmed_end(self):
        if self.end > self.start and self.data[self.end - 1] == 0x0D:
            return self.end - 1
        return self.end

    def as_bytes(self):
        return bytes(self.data[self.start:self._trimmed_end()])

    def field_count(self):
        return len(self.seps) + 1

    def field_span(self, i):
        if i > len(self.seps):
            return None
        a = self.start if i == 0 else int(self.seps[i - 1]) + 1
        b = self._trimmed_end() if i == len(self.seps) else int(self.seps[i])
        return (a, b)

    def field_raw(self, i):
        sp = self.field_span(i)
        return None if sp is None else bytes(self.data[sp[0]:sp[1]])

    def field(self, i):
        raw = self.field_raw(i)
        return None if raw is None else clean(raw)

    def fields(self):
        return [self.field(i) for i in range(self.field_count())]

    def fields_raw(self):
        return [self.field_raw(i) for i in range(self.field_count())]


def clean(raw):
    """Strip outer quotes and collapse doubled quotes (csv_geo.rs:875-895)."""
    if len(raw) >= 2 and raw[0] == 0x22 and raw[-1] == 0x22:
        inner = raw[1:-1]
        if b'"' not in inner:
            return inner
        out = bytearray()
        i = 0
        while i < len(inner):
            out.append(inner[i])
            i += 2 if (inner[i] == 0x22 and i + 1 < len(inner) and inner[i + 1] == 0x22) else 1
        return bytes(out)
    return raw


class Parsed:
    """Tape over borrowed input (csv_geo.rs:415-466): separator offsets and
    record ends `(separators_before << 32) | terminator_offset`."""

    def __init__(self, data, seps, ends, dialect):
        self.data = data
        self.seps = seps
        self.ends = ends
        self.dialect = dialect

    def terminated_record_count(self):
        return len(self.ends)

    def records(self):
        return self.records_range(0, len(self.ends))

    def records_range(self, lo, hi):
        data, seps, ends = self.data, self.seps, self.ends
        n = len(data)
        if lo == 0:
            byte_pos, sep_pos = 0, 0
        else:
            prev = int(ends[lo - 1])
            byte_pos, sep_pos = (prev & 0xFFFFFFFF) + 1, prev >> 32
        if lo >= hi and len(ends):
            data_end = byte_pos
        elif hi == len(ends):
            data_end = n
        else:
            data_end = (int(ends[hi - 1]) & 0xFFFFFFFF) + 1
        k = lo
        while True:
            start = byte_pos
            if k < hi:
                e = int(ends[k])
                k += 1
                end, cum = e & 0xFFFFFFFF, e >> 32
                rs = seps[sep_pos:cum]
                sep_pos = cum
                byte_pos = end + 1
            else:
                if start >= data_end:
                    return
                rs = seps[sep_pos:]
                sep_pos = len(seps)
                byte_pos = data_end
                end = data_end
            # csv_hash skips comment records (csv_hash.rs:547-557)
            if self.dialect == CSV_HASH and end > start and data[start] == 0x23:
                continue
            yield Record(data, start, end, rs)


def bitmap_get(bitmap, row):
    """Bit `row` of an LSB-first validity bitmap (csv_geo.rs:1105)."""
    return (int(bitmap[row >> 6]) >> (row & 63)) & 1 != 0


def string_at(offsets, data, row):
    """Row `row` of a string column (csv_hash.rs:1444)."""
    return bytes(data[int(offsets[row]):int(offsets[row + 1])])


_engine = None


def engine(device=0):
    """The process-wide default engine."""
    global _engine
    if _engine is None:
        _engine = Engine(device)
    return _engine


def _host_bytes(data):
    if isinstance(data, (bytes, bytearray, memoryview)):
        return bytes(data)
    if isinstance(data, np.ndarray):
        return data.tobytes()
    return data.cpu().numpy().tobytes()


def index_structurals(data, dialect=CSV):
    """Offsets of every structural byte (u32 NumPy array)."""
    return engine().index_structurals(data, dialect).cpu().numpy().view(np.uint32)


def index_structurals_par(data, threads=1, dialect=CSV):
    return index_structurals(data, dialect)


def parse(data, dialect=CSV):
    seps, ends = engine().parse_tape(data, dialect)
    return Parsed(_host_bytes(data), seps.cpu().numpy().view(np.uint32), ends.cpu().numpy().view(np.uint64),
                  dialect)


def parse_par(data, threads=1, dialect=CSV):
    return parse(data, dialect)


def parse_into(data, recycle, dialect=CSV):
    """Like parse, writing the tape into the device buffers of an earlier
    Parsed (csv_geo.rs:405 parse_into: the tape allocations are recycled,
    their contents discarded)."""
    reuse = getattr(recycle, "_device", None) if recycle is not None else None
    seps, ends = engine().parse_tape(data, dialect, reuse=reuse)
    p = Parsed(_host_bytes(data), seps.cpu().numpy().view(np.uint32), ends.cpu().numpy().view(np.uint64), dialect)
    # keep the whole device buffers (the tape tensors are views of them) for the next recycle
    p._device = tuple(t._base if t._base is not None else t for t in (seps, ends))
    return p


def parse_columns(data, schema):
    return engine().parse_columns(data, schema)


def parse_columns_par(data, threads, schema):
    return parse_columns(data, schema)


def parse_columns_chunks_par(data, threads, schema):
    return [parse_columns(data, schema)]


def parse_csv_geo_stats(data, dialect=CSV, fields=(4, 5)):
    return engine().stats_count_sum(data, dialect, fields[0], fields[1])


def parse_csv_geo_stats_par(data, threads=1, dialect=CSV, fields=(4, 5)):
    return parse_csv_geo_stats(data, dialect, fields)


def parse_csv_geo_text_stats(data, dialect=CSV, fields=(1, 4, 5)):
    return engine().geo_text_stats(data, dialect, fields)


def parse_csv_geo_text_stats_par(data, threads=1, dialect=CSV, fields=(1, 4, 5)):
    return parse_csv_geo_text_stats(data, dialect, fields)


def parse_field_bytes(data, dialect=CSV_HASH):
    return engine().field_bytes(data, dialect)


def parse_field_bytes_par(data, threads=1, dialect=CSV_HASH):
    return parse_field_bytes(data, dialect)


def parse_ndjson_id_score(data):
    return engine().ndjson_id_score(data)


def parse_ndjson_id_score_par(data, threads=1):
    return parse_ndjson_id_score(data)
