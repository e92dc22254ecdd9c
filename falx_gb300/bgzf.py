"""bgzf streams: a writer (for inputs and tests) and the GPU path that
inflates every block on the device and parses the text where it lands
(bgzf.rs:61 scan, :201 decompress, :538 parse_gz_par;
examples/gpu_pipeline.rs:1-8).

A bgzf stream is a series of gzip members of at most 64 KiB each: a
header whose extra field holds the `BC` subfield with the member's size
less one (BSIZE), a raw DEFLATE payload, then CRC32 and ISIZE (the
uncompressed size), ending with an empty member."""

import struct
import zlib
from concurrent.futures import ThreadPoolExecutor
from ctypes import byref, c_uint64, c_void_p

import numpy as np

from . import _lib
from ._lib import check

BLOCK_DATA = 0xFF00  # uncompressed bytes per member, as bgzip writes them
EOF_MEMBER = bytes.fromhex("1f8b08040000000000ff0600424302001b0003000000000000000000")
GZ_BLOCK = np.dtype([("in_off", "<u8"), ("out_off", "<u8"), ("in_len", "<u4"), ("out_len", "<u4")])


def _member(chunk, level):
    if level == 0:
        # stored blocks only
        c = zlib.compressobj(0, zlib.DEFLATED, -15)
    else:
        c = zlib.compressobj(level, zlib.DEFLATED, -15, 9, zlib.Z_DEFAULT_STRATEGY)
    payload = c.compress(chunk) + c.flush()
    bsize = 12 + 6 + len(payload) + 8 - 1
    head = struct.pack("<BBBBIBBH", 0x1F, 0x8B, 8, 4, 0, 0, 0xFF, 6) + b"BC" + struct.pack("<HH", 2, bsize)
    return head + payload + struct.pack("<II", zlib.crc32(chunk), len(chunk))


def compress(data, level=6, block=BLOCK_DATA, threads=8):
    """bgzf bytes of `data` (members compressed in parallel by zlib)."""
    mv = memoryview(bytes(data) if not isinstance(data, (bytes, bytearray)) else data)
    chunks = [mv[i: i + block] for i in range(0, len(mv), block)]
    with ThreadPoolExecutor(max(1, threads)) as ex:
        members = list(ex.map(lambda c: _member(bytes(c), level), chunks))
    return b"".join(members) + EOF_MEMBER


def scan(comp):
    """The non-empty members (structured array in_off, out_off, in_len,
    out_len) and the inflated length (falx_bgzf_scan)."""
    lib = _lib.load()
    a = np.frombuffer(memoryview(comp), dtype=np.uint8) if not isinstance(comp, np.ndarray) else comp
    n, total = c_uint64(), c_uint64()
    rc = lib.falx_bgzf_scan(a.ctypes.data_as(c_void_p), a.size, None, 0, byref(n), byref(total))
    if rc not in (_lib.FALX_OK, _lib.FALX_ERR_CAPACITY):
        check(rc, "falx_bgzf_scan")
    blocks = np.zeros(max(n.value, 1), dtype=GZ_BLOCK)
    check(lib.falx_bgzf_scan(a.ctypes.data_as(c_void_p), a.size, blocks.ctypes.data_as(c_void_p), n.value,
                             byref(n), byref(total)), "falx_bgzf_scan")
    return blocks[: n.value], total.value


def inflate(engine, comp, blocks=None, total=None, out=None, status=False):
    """Inflate a bgzf stream on the GPU: returns the device uint8 tensor of
    the text (and the per-block status array when status=True). `comp` may
    be host bytes (copied in) or a device tensor; `blocks`/`total` from
    scan() when already known."""
    torch = engine.torch
    if blocks is None:
        host = comp.cpu().numpy() if isinstance(comp, torch.Tensor) else comp
        blocks, total = scan(host)
    d = engine.to_device(comp)
    engine._sync_stream()
    if out is None:
        out = engine.empty(max(total, 1), torch.uint8)
    st = np.zeros(max(len(blocks), 1), dtype=np.int32)
    failed = c_uint64()
    rc = engine.lib.falx_bgzf_inflate(engine.ctx, c_void_p(d.data_ptr()), d.numel(),
                                      blocks.ctypes.data_as(c_void_p), len(blocks), c_void_p(out.data_ptr()),
                                      out.numel(), st.ctypes.data_as(c_void_p), byref(failed))
    if status:
        if rc not in (_lib.FALX_OK, _lib.FALX_ERR_FORMAT):
            check(rc, "falx_bgzf_inflate")
        return out[:total], st[: len(blocks)]
    check(rc, "falx_bgzf_inflate")
    return out[:total]


def parse_gz(engine, comp, schema, stats_fields=None):
    """Inflate on the GPU, then one falx_parse over the text in place
    (parse_gz_par, bgzf.rs:538: here the whole stream is one run of
    records, so there is one result rather than one per worker)."""
    text = inflate(engine, comp)
    return engine.parse_all(text, schema, stats_fields=stats_fields)
