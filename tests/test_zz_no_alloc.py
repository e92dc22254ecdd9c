"""The allocation-free structural index (falx_index_structurals_noalloc).

It serves callers that may not allocate device memory (a full or frozen
memory pool, a host application that owns every allocation); it keeps its
look-back scratch in a fixed array inside the library. Checked through the
C ABI against the regular entry point, on two calls in a row so the second
call runs over the scratch the first one left behind. The file sorts last so
a run that stops at its first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, data, dialect, cap):
    import torch

    out = torch.empty(max(cap, 1), dtype=torch.int32, device="cuda")
    n = ctypes.c_uint64()
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.falx_index_structurals_noalloc(torch.cuda.current_device(), dialect, ctypes.c_void_p(data.data_ptr()),
                                            data.numel(), ctypes.c_void_p(out.data_ptr()), cap, ctypes.byref(n),
                                            ctypes.c_void_p(stream))
    return rc, out[: n.value].cpu().numpy().view(np.uint32)


def test_noalloc_index_matches_regular_entry_point():
    import torch

    import falx_gb300 as fx
    from falx_gb300 import _lib, gen

    lib = _lib.load()
    eng = fx.Engine(0)
    docs = [(gen.generate(gen.CSV_HASH, 24 << 20), fx.CSV_HASH), (gen.generate(gen.ADVERSARIAL, 8 << 20), fx.CSV_HASH),
            (gen.generate(gen.CSV_GEO, 5 << 20), fx.CSV), (gen.generate(gen.NDJSON, 3 << 20), fx.NDJSON)]
    for host, dialect in docs:
        data = torch.from_numpy(host.copy()).cuda()
        want = eng.index_structurals(data, dialect).cpu().numpy().view(np.uint32)
        for call in range(2):
            rc, got = _noalloc(lib, data, dialect, want.size + 16)
            assert rc == _lib.FALX_OK, (call, rc)
            assert np.array_equal(got, want), call
        # a misaligned view of the same buffer
        sub = data[3:]
        want = eng.index_structurals(sub, dialect).cpu().numpy().view(np.uint32)
        rc, got = _noalloc(lib, sub, dialect, want.size + 16)
        assert rc == _lib.FALX_OK and np.array_equal(got, want)
    eng.close()


def test_noalloc_rejects_inputs_over_its_limit():
    import torch

    from falx_gb300 import _lib

    lib = _lib.load()
    small = torch.zeros(16, dtype=torch.uint8, device="cuda")
    out = torch.empty(4, dtype=torch.int32, device="cuda")
    n = ctypes.c_uint64()
    # the length is checked before any device access
    rc = lib.falx_index_structurals_noalloc(torch.cuda.current_device(), 1, ctypes.c_void_p(small.data_ptr()),
                                            _lib.NOALLOC_MAX_BYTES + 1, ctypes.c_void_p(out.data_ptr()), 4,
                                            ctypes.byref(n), None)
    assert rc == _lib.FALX_ERR_INPUT_TOO_LARGE
    # capacity shortfall reports the count, like the regular entry point
    doc = torch.from_numpy(np.frombuffer(b"a,b\nc,d\n" * 64, dtype=np.uint8).copy()).cuda()
    rc = lib.falx_index_structurals_noalloc(torch.cuda.current_device(), 0, ctypes.c_void_p(doc.data_ptr()),
                                            doc.numel(), ctypes.c_void_p(out.data_ptr()), 4, ctypes.byref(n), None)
    assert rc == _lib.FALX_ERR_CAPACITY and n.value == 256


def test_noalloc_allocates_nothing():
    """After one warm-up call per dialect, calls of different sizes leave the
    device's free memory unchanged."""
    import torch

    import falx_gb300 as fx
    from falx_gb300 import _lib, gen

    lib = _lib.load()
    docs = [(gen.generate(gen.CSV_HASH, 7 << 20), fx.CSV_HASH), (gen.generate(gen.CSV_GEO, 3 << 20), fx.CSV),
            (gen.generate(gen.NDJSON, 1 << 20), fx.NDJSON), (gen.generate(gen.CSV_HASH, 40 << 20), fx.CSV_HASH)]
    dev = [torch.from_numpy(h.copy()).cuda() for h, _ in docs]
    outs = [torch.empty(d.numel() // 2 + 64, dtype=torch.int32, device="cuda") for d in dev]
    stream = torch.cuda.current_stream().cuda_stream
    n = ctypes.c_uint64()

    def call(k, length=None):
        d = dev[k]
        rc = lib.falx_index_structurals_noalloc(torch.cuda.current_device(), docs[k][1], ctypes.c_void_p(d.data_ptr()),
                                                d.numel() if length is None else min(length, d.numel()),
                                                ctypes.c_void_p(outs[k].data_ptr()), outs[k].numel(), ctypes.byref(n),
                                                ctypes.c_void_p(stream))
        assert rc == _lib.FALX_OK, rc
        return n.value

    for k in range(len(docs)):
        call(k)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    counts = [call(k, length) for k in (3, 0, 1, 2, 3) for length in (None, 12345, 1 << 20)]
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert all(c > 0 for c in counts)


_WRAP_CHILD = r"""
import ctypes, sys
import numpy as np, torch
import falx_gb300 as fx
from falx_gb300 import _lib, gen
lib = _lib.load()
eng = fx.Engine(0)
for host, dialect in [(gen.generate(gen.CSV_HASH, 9 << 20), fx.CSV_HASH), (gen.generate(gen.CSV_GEO, 2 << 20), fx.CSV)]:
    data = torch.from_numpy(host.copy()).cuda()
    want = eng.index_structurals(data, dialect).cpu().numpy().view(np.uint32)
    out = torch.empty(want.size + 16, dtype=torch.int32, device="cuda")
    for call in range(3):
        n = ctypes.c_uint64()
        rc = lib.falx_index_structurals_noalloc(0, dialect, ctypes.c_void_p(data.data_ptr()), data.numel(),
                                                ctypes.c_void_p(out.data_ptr()), out.numel(), ctypes.byref(n), None)
        got = out[: n.value].cpu().numpy().view(np.uint32)
        if rc != 0 or not np.array_equal(got, want):
            print("mismatch", dialect, call, rc, n.value, want.size)
            sys.exit(1)
eng.close()
print("ok")
"""


def test_noalloc_epoch_wrap():
    """Started two calls before the epoch wraps: the third call clears the
    whole status array and restarts at epoch 1; every call still matches the
    regular entry point."""
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, FALX_NOALLOC_EPOCH_START=str((1 << 28) - 3))
    r = subprocess.run([sys.executable, "-c", _WRAP_CHILD], cwd=root, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr
