"""The columns kernel's word-at-a-time decoders (swar.cuh), built for the
host and checked against str::parse semantics (Python's int / float are
exact and correctly rounded) on boundary shapes and random cells, with
arbitrary bytes after each cell."""

import ctypes
import os
import random
import re
import struct
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
U32_RE = re.compile(rb"[0-9]{1,10}")
FIXED6_RE = re.compile(rb"[+-]?[0-9]{1,3}\.[0-9]{6}")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("swar") / "libswar_host.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "falx_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "swar_host.cpp"), "-o", out], check=True)
    l = ctypes.CDLL(out)
    l.swar_u32_cell.argtypes = [ctypes.c_char_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
    l.swar_fixed6_cell.argtypes = [ctypes.c_char_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64),
                                   ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int)]
    return l


def cells(rng):
    fixed = [b"0", b"7", b"12345678", b"00000001", b"123456789", b"+5", b"-5", b"1a", b"a1", b"1234567a", b"/", b":",
             b"\x80", b"\xba1", b"1\xff", b"0.000000", b"-0.000000", b"+0.000001", b"1.500000", b"-172.432059",
             b"999.999999", b"1000.000000", b"1.5", b"12.3456789", b".123456", b"-.123456", b"1.23456a",
             b"1a.123456", b"+-1.000000", b"1.1234567", b"12.123456", b"123.12345", b"89.999999", b"1:.123456",
             b"4294967295", b"4294967296", b"9999999999", b"0000000000", b"0004294967", b"2147483648", b"a234567890",
             b"123456789a", b"12345678901", b"1234\xba67890", b"\xba23456789", b"12345678\xba",
             b"1/.123456", b"\xba.123456", b"1.12345\xba", b"1,000000", b"", b"12.12345."]
    out = list(fixed)
    alphabet = b"0123456789.+-a/:\xba\x80 "
    for _ in range(20000):
        kind = rng.random()
        if kind < 0.4:
            s = (rng.choice([b"", b"-", b"+"]) + bytes(rng.choice(b"0123456789") for _ in range(rng.randint(1, 3)))
                 + b"." + bytes(rng.choice(b"0123456789") for _ in range(6)))
        elif kind < 0.7:
            s = bytes(rng.choice(b"0123456789") for _ in range(rng.randint(1, 11)))
        else:
            s = bytes(rng.choice(alphabet) for _ in range(rng.randint(0, 11)))
        if rng.random() < 0.1 and s:  # one corrupted byte
            i = rng.randrange(len(s))
            s = s[:i] + bytes([rng.randrange(256)]) + s[i + 1:]
        out.append(s)
    return out


def test_u32_and_fixed6_match_str_parse(lib):
    rng = random.Random(0x5A5A)
    v = ctypes.c_uint32()
    bits, m, neg = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_int()
    accepted = [0, 0]
    for s in cells(rng):
        buf = s + bytes(rng.randrange(256) for _ in range(8))  # whatever follows the cell
        ok = lib.swar_u32_cell(buf, len(s), ctypes.byref(v))
        assert ok == bool(U32_RE.fullmatch(s) and int(s) <= 0xFFFFFFFF), s
        if ok:
            accepted[0] += 1
            assert v.value == int(s), s
        ok = lib.swar_fixed6_cell(buf, len(s), ctypes.byref(bits), ctypes.byref(m), ctypes.byref(neg))
        assert ok == bool(FIXED6_RE.fullmatch(s)), s
        if ok:
            accepted[1] += 1
            assert bits.value == struct.unpack("<Q", struct.pack("<d", float(s)))[0], s
            assert m.value == int(s.lstrip(b"+-").replace(b".", b"")), s
            assert neg.value == s.startswith(b"-"), s
    assert min(accepted) > 1000
