"""The C-ABI library loads without a GPU and exports every entry point that
include/falx_gpu.h declares."""

import ctypes
import os
import re

from falx_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            syms |= set(re.findall(r"\b(falx_[a-z0-9_]+)\s*\(", text))
    return syms


def test_library_exports_every_declared_symbol():
    build.build_gpu()
    lib = ctypes.CDLL(build.GPU_LIB)
    syms = declared_symbols()
    assert len(syms) >= 13
    for s in sorted(syms):
        assert hasattr(lib, s), s


def test_bindings_cover_header():
    assert declared_symbols() == set(_lib.SIGNATURES)


def test_strerror_without_gpu():
    lib = _lib.load()
    assert lib.falx_strerror(_lib.FALX_ERR_CAPACITY) == b"output capacity too small"
