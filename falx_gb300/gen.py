"""Seeded synthetic inputs (csrc/gen.c): identical bytes on every host."""

import ctypes
import os

import numpy as np

from . import build

CSV_GEO, CSV_HASH, NDJSON, TSV, LOGFMT, ADVERSARIAL = 0, 1, 2, 3, 4, 5

# Per-format seeds of the reference's dataset generator
# (examples/make_datasets.rs:221-232) where the family matches.
SEEDS = {CSV_GEO: 0xDEADBEEFCAFEBABE, CSV_HASH: 0xC0FFEE15600DF00D, NDJSON: 0x853C49E6748FEA9B,
         TSV: 0xA0761D6478BD642F, LOGFMT: 0xE7037ED1A0B428DB, ADVERSARIAL: 0x5EEDC5A51234ABCD}

_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build.build_gen())
        lib.falx_gen.restype = ctypes.c_uint64
        lib.falx_gen.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                                 ctypes.c_int]
        _lib = lib
    return _lib


def generate(kind, target_bytes, seed=None, threads=None, out=None):
    """About `target_bytes` of document `kind` as a uint8 array. `out` may be
    a preallocated (e.g. pinned) uint8 array; the document is written there."""
    lib = _load()
    seed = SEEDS[kind] if seed is None else seed
    threads = threads or os.cpu_count() or 1
    cap = target_bytes + (1 << 20)
    buf = out if out is not None else np.empty(cap, dtype=np.uint8)
    n = lib.falx_gen(kind, seed, target_bytes, buf.ctypes.data_as(ctypes.c_void_p), buf.size, threads)
    if n > buf.size:
        raise ValueError("output buffer too small: need %d bytes" % n)
    return buf[:n]
