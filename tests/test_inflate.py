"""bgzf / raw DEFLATE on the CPU: the oracle's serial decoder and a host
build of the GPU decoder's core (inflate_core.h, under AddressSanitizer)
against zlib's output and against each other, including corrupt streams
(bit flips, truncations, wrong sizes): both must accept and reject the same
streams, agree byte for byte when they accept, and never read or write out
of bounds. The bgzf member walk is checked on well-formed and malformed
framing (bgzf.rs:61-108)."""

import os
import random
import struct
import subprocess
import zlib

import numpy as np
import pytest

import oracle
from falx_gb300 import bgzf, gen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def raw_deflate(data, level=6, strategy=zlib.Z_DEFAULT_STRATEGY):
    c = zlib.compressobj(level, zlib.DEFLATED, -15, 9, strategy)
    return c.compress(data) + c.flush()


def fnv(b):
    h = 1469598103934665603
    for x in b:
        h = ((h ^ x) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def samples():
    rng = random.Random(20261204)
    text = bytes(gen.generate(gen.CSV_HASH, 300 << 10))[:200000]
    out = [b"", b"a", b"abc" * 1000, bytes(range(256)) * 40, bytes(rng.getrandbits(8) for _ in range(5000)),
           text[:65280], text[1000:1100], b"\x00" * 65280]
    return out


def streams():
    """(payload, original) pairs over levels and strategies: stored, fixed
    and dynamic blocks, runs (overlapping matches), long distances."""
    res = []
    for data in samples():
        for level in (0, 1, 6, 9):
            res.append((raw_deflate(data, level), data))
        res.append((raw_deflate(data, 6, zlib.Z_FIXED), data))
        res.append((raw_deflate(data, 6, zlib.Z_HUFFMAN_ONLY), data))
        res.append((raw_deflate(data, 6, zlib.Z_RLE), data))
    return res


@pytest.fixture(scope="module")
def fuzz_bin(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("inflate") / "inflate_fuzz")
    cmd = ["g++", "-O1", "-g", "-std=c++17", "-DGZ_FUZZ_MAIN", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=all", "-I", os.path.join(ROOT, "falx_gb300", "csrc"),
           os.path.join(ROOT, "tests", "inflate_host.cpp"), "-o", out]
    if subprocess.run(cmd, capture_output=True).returncode != 0:
        cmd = [c for c in cmd if not c.startswith("-fsanitize") and c != "-fno-sanitize-recover=all"]
        subprocess.run(cmd, check=True)
    return out


def run_core(fuzz_bin, tmp_path, cases):
    path = str(tmp_path / "cases.bin")
    with open(path, "wb") as f:
        for payload, n in cases:
            f.write(struct.pack("<II", len(payload), n) + payload)
    r = subprocess.run([fuzz_bin, path], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return [(int(a), int(b, 16)) for a, b in (line.split() for line in r.stdout.splitlines())]


def test_oracle_matches_zlib():
    for payload, data in streams():
        rc, out = oracle.inflate(payload, len(data))
        assert rc == 0 and out == data
        assert zlib.decompress(payload, -15) == data


def test_core_matches_zlib(fuzz_bin, tmp_path):
    cases = streams()
    got = run_core(fuzz_bin, tmp_path, [(p, len(d)) for p, d in cases])
    for (rc, h), (p, d) in zip(got, cases):
        assert rc == 0 and h == fnv(d)


def corruptions(rng, payload, n):
    out = []
    for _ in range(6):
        b = bytearray(payload)
        if b:
            for _ in range(rng.randint(1, 3)):
                i = rng.randrange(len(b))
                b[i] ^= 1 << rng.randrange(8)
        out.append((bytes(b), n))
    if payload:
        out.append((payload[: rng.randrange(len(payload))], n))  # truncated
    out.append((payload, n + 1))                                 # ISIZE too large
    out.append((payload, max(n - 1, 0)))                         # ISIZE too small
    out.append((bytes(rng.getrandbits(8) for _ in range(rng.randint(0, 300))), rng.randint(0, 5000)))
    return out


def test_core_and_oracle_agree_on_corrupt_streams(fuzz_bin, tmp_path):
    rng = random.Random(7)
    cases = []
    for payload, data in streams():
        cases += corruptions(rng, payload, len(data))
    got = run_core(fuzz_bin, tmp_path, cases)
    accepted = 0
    for (rc, h), (p, n) in zip(got, cases):
        orc, out = oracle.inflate(p, n)
        assert (rc == 0) == (orc == 0), (rc, orc)
        if rc == 0:
            accepted += 1
            assert h == fnv(out)
    assert accepted < len(cases)


def test_bgzf_scan_and_inflate_par():
    data = bytes(gen.generate(gen.CSV_HASH, 3 << 20))
    comp = bgzf.compress(data, 6)
    blocks, total = oracle.bgzf_scan(comp)
    assert total == len(data) and len(blocks) == (len(data) + bgzf.BLOCK_DATA - 1) // bgzf.BLOCK_DATA
    out, st = oracle.bgzf_inflate_par(comp, 4)
    assert not st.any() and out.tobytes() == data
    # the package's scan (the C ABI's host walk) agrees with the oracle's
    pb, ptotal = bgzf.scan(comp)
    assert ptotal == total and np.array_equal(pb.view(np.uint8), blocks.view(np.uint8))


def test_bgzf_malformed_framing():
    from falx_gb300 import FalxError

    good = bgzf.compress(b"x,y\n" * 1000)
    for bad in (good[:5], b"\x1f\x8b\x08\x00" + good[4:], good[:-3], b"\x00" + good[1:]):
        assert oracle.bgzf_scan(bad)[0] is None
        with pytest.raises(FalxError):
            bgzf.scan(bad)
    assert bgzf.scan(bgzf.EOF_MEMBER)[1] == 0
    assert bgzf.scan(b"")[1] == 0
