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
