"""The tile index kernel (FALX_INDEX_KERNEL=tile, read when a context is
created: plain scans use `index_kernel` instead of the index pass) gives
the same outputs as the default index pass, through the host-buffer entry
point at a size that would take the pipelined form (which needs the index
pass, so the tile kernel runs the whole-input form) and through the device
entry points."""

import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

DIGEST = r"""
import hashlib, sys
import numpy as np
sys.path.insert(0, {root!r}); sys.path.insert(0, {here!r})
import falx_gb300 as fx
from falx_gb300 import gen
from test_parse_host import COLS, parse_host

def digest(eng):
    h = hashlib.sha256()
    doc = gen.generate(gen.CSV_HASH, 72 << 20).tobytes()
    index, rows, keep, str_len = parse_host(eng, doc, fx.CSV_HASH, COLS)
    h.update(index.tobytes()); h.update(str(rows).encode())
    for (v, valid, sd), sl in zip(keep, str_len):
        h.update(v[: rows + 1].tobytes()); h.update(valid[: (rows + 63) // 64].tobytes())
        if sd is not None:
            h.update(sd[:sl].tobytes())
    small = gen.generate(gen.CSV_GEO, 4 << 20)
    h.update(eng.index_structurals(small, fx.CSV).cpu().numpy().tobytes())
    got = eng.parse_columns(small, fx.Schema(fx.CSV, [(0, fx.U32), (1, fx.STR), (4, fx.F64)]))
    h.update(str(got.rows).encode())
    for k in range(3):
        for part in got.host(k).values():
            h.update(part if isinstance(part, bytes) else np.asarray(part).tobytes())
    return h.hexdigest()

print(digest(fx.Engine(0)))
"""


def run_digest(env_extra):
    env = dict(os.environ)
    env.update(env_extra)
    code = DIGEST.format(root=ROOT, here=HERE)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout.strip().splitlines()[-1]


def test_tile_index_kernel_matches_index_pass():
    plain = run_digest({"FALX_INDEX_KERNEL": "pass"})
    tile = run_digest({"FALX_INDEX_KERNEL": "tile"})
    assert tile == plain
