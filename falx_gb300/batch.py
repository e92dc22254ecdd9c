"""Batched documents (falx_batch_*): many documents of uneven sizes parsed
in one persistent launch replayed from a CUDA graph.

A batch holds, per document, its structural index and its two f64 columns
(latitude / longitude of the geo schemas) with validity, in three device
arenas; documents start 256-byte aligned in one device buffer.
"""

import ctypes
import math
import os
from concurrent.futures import ThreadPoolExecutor
from ctypes import byref, c_float, c_uint32, c_uint64, c_void_p

import numpy as np

from . import _lib, gen
from ._lib import CSV, LOGFMT, TSV, check

# The geo documents' lat / lon field ordinals per dialect (logfmt fields
# alternate key and value: lat and lon are value fields 9 and 11).
GEO_FIELDS = {CSV: (4, 5), TSV: (4, 5), LOGFMT: (9, 11)}
KIND_OF = {CSV: gen.CSV_GEO, TSV: gen.TSV, LOGFMT: gen.LOGFMT}
ALIGN = 256


def mixed_sizes(ndocs, total_bytes, lo=4 << 10, hi=64 << 20, seed=0xBA7C4):
    """Document sizes drawn log-uniform in [lo, hi], then scaled so they sum
    to about total_bytes (never below lo)."""
    rng = np.random.default_rng(seed)
    s = np.exp(rng.uniform(math.log(lo), math.log(hi), ndocs))
    s *= total_bytes / s.sum()
    return np.maximum(s, lo).astype(np.int64)


def mixed_dialects(ndocs, seed=0xBA7C5):
    """50% CSV, 25% TSV, 25% logfmt, shuffled."""
    rng = np.random.default_rng(seed)
    d = np.array([CSV] * (ndocs // 2) + [TSV] * (ndocs // 4) + [LOGFMT] * (ndocs - ndocs // 2 - ndocs // 4))
    rng.shuffle(d)
    return d


def generate(sizes, dialects, seed=0xD0C5, out=None):
    """Documents into one host buffer: (buffer, offsets, lengths)."""
    offs, pos = [], 0
    for s in sizes:
        offs.append(pos)
        pos += (int(s) + ALIGN - 1) // ALIGN * ALIGN + ALIGN
    buf = out if out is not None else np.zeros(pos + (2 << 20), dtype=np.uint8)

    def one(k):
        s, d = int(sizes[k]), int(dialects[k])
        cap = (s + ALIGN - 1) // ALIGN * ALIGN + ALIGN
        doc = gen.generate(KIND_OF[d], s, seed=seed + k, threads=1, out=np.empty(s + (1 << 20), dtype=np.uint8))
        n = min(doc.size, cap)
        buf[offs[k]: offs[k] + n] = doc[:n]
        return n

    # the generator releases the GIL: documents are written in parallel
    with ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        lens = list(ex.map(one, range(len(sizes))))
    return buf, np.array(offs, dtype=np.int64), np.array(lens, dtype=np.int64)


class Batch:
    """A planned batch on an Engine. `data` is a device uint8 tensor holding
    the documents at `offsets` (16-byte aligned) with `lens` and `dialects`."""

    def __init__(self, engine, data, offsets, lens, dialects, config=None, fields=None):
        torch = engine.torch
        self.engine = engine
        self.data = data
        self.n = len(lens)
        self.lens = np.asarray(lens, dtype=np.int64)
        self.dialects = np.asarray(dialects, dtype=np.int64)
        icaps = self.lens // 3 + 64
        rcaps = self.lens // 16 + 64
        self.ioff = np.concatenate([[0], np.cumsum(icaps)]).astype(np.int64)
        self.roff = np.concatenate([[0], np.cumsum(rcaps)]).astype(np.int64)
        woff = np.concatenate([[0], np.cumsum((rcaps + 63) // 64)]).astype(np.int64)
        self.woff = woff
        dev = data.device
        self.index = torch.empty(int(self.ioff[-1]) + 1, dtype=torch.int32, device=dev)
        self.col0 = torch.empty(int(self.roff[-1]) + 1, dtype=torch.float64, device=dev)
        self.col1 = torch.empty(int(self.roff[-1]) + 1, dtype=torch.float64, device=dev)
        self.valid0 = torch.empty(int(woff[-1]) + 1, dtype=torch.int64, device=dev)
        self.valid1 = torch.empty(int(woff[-1]) + 1, dtype=torch.int64, device=dev)
        docs = (_lib.falx_doc * max(self.n, 1))()
        base = data.data_ptr()
        for k in range(self.n):
            d = int(self.dialects[k])
            f0, f1 = (fields or GEO_FIELDS)[d]
            x = docs[k]
            x.data = base + int(offsets[k])
            x.len = int(self.lens[k])
            x.dialect = d
            x.field0, x.field1 = f0, f1
            x.index = self.index.data_ptr() + 4 * int(self.ioff[k])
            x.index_cap = int(icaps[k])
            x.col0 = self.col0.data_ptr() + 8 * int(self.roff[k])
            x.col1 = self.col1.data_ptr() + 8 * int(self.roff[k])
            x.valid0 = self.valid0.data_ptr() + 8 * int(woff[k])
            x.valid1 = self.valid1.data_ptr() + 8 * int(woff[k])
            x.rows_cap = int(rcaps[k])
        self.docs = docs
        engine._sync_stream()
        ptr = c_void_p()
        cfg = None
        if config is not None:
            cfg = _lib.falx_batch_config(*config)
        check(engine.lib.falx_batch_create(engine.ctx, docs, self.n, byref(cfg) if cfg else None, byref(ptr)),
              "falx_batch_create")
        self.ptr = ptr

    def run(self):
        check(self.engine.lib.falx_batch_run(self.ptr, self.docs), "falx_batch_run")

    def info(self):
        cfg = _lib.falx_batch_config()
        items, grid, graph = c_uint32(), c_uint32(), ctypes.c_int()
        check(self.engine.lib.falx_batch_info(self.ptr, byref(cfg), byref(items), byref(grid), byref(graph)),
              "falx_batch_info")
        return {"chunk_bytes": cfg.chunk_bytes, "ctas_per_sm": cfg.ctas_per_sm, "staging": cfg.staging,
                "items": items.value, "grid": grid.value, "graph": bool(graph.value)}

    def result(self, k):
        """(index uint32, col0 f64, valid0 words, col1, valid1) of document k (host)."""
        x = self.docs[k]
        i0, r0, w0 = int(self.ioff[k]), int(self.roff[k]), int(self.woff[k])
        rows = int(x.rows)
        words = (rows + 63) // 64
        idx = self.index[i0: i0 + int(x.n_index)].cpu().numpy().view(np.uint32)
        c0 = self.col0[r0: r0 + rows].cpu().numpy()
        c1 = self.col1[r0: r0 + rows].cpu().numpy()
        v0 = self.valid0[w0: w0 + words].cpu().numpy().view(np.uint64)
        v1 = self.valid1[w0: w0 + words].cpu().numpy().view(np.uint64)
        return idx, c0, v0, c1, v1

    def close(self):
        if self.ptr:
            self.engine.lib.falx_batch_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune(engine, batch):
    """Autotune on `batch`'s documents; the context keeps the result."""
    best = _lib.falx_batch_config()
    ms = c_float()
    check(engine.lib.falx_batch_tune(engine.ctx, batch.docs, batch.n, byref(best), byref(ms)), "falx_batch_tune")
    return {"chunk_bytes": best.chunk_bytes, "ctas_per_sm": best.ctas_per_sm, "staging": best.staging,
            "ms": ms.value}


def plan(lens, chunk_bytes):
    """The work queue falx_batch_create would build: [(doc, tile_lo, tile_hi)]."""
    lib = _lib.load()
    lens = np.ascontiguousarray(lens, dtype=np.uint64)
    n = c_uint32()
    check(lib.falx_batch_plan(c_void_p(lens.ctypes.data), lens.size, chunk_bytes, None, 0, byref(n)), "plan")
    items = np.zeros(max(3 * n.value, 3), dtype=np.uint32)
    check(lib.falx_batch_plan(c_void_p(lens.ctypes.data), lens.size, chunk_bytes, c_void_p(items.ctypes.data),
                              n.value, byref(n)), "plan")
    return [tuple(int(v) for v in items[3 * k: 3 * k + 3]) for k in range(n.value)]
