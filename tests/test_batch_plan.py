"""The batched launch's work queue (host planner, no GPU): every tile of
every document exactly once, tiles of a document in order, large documents
tile by tile first, whole documents after them largest first."""

import numpy as np

from falx_gb300 import batch

TILE = 16384


def test_plan_covers_every_tile_in_order():
    rng = np.random.default_rng(3)
    lens = np.concatenate([[0, 1, TILE, TILE + 1, 5 << 20], rng.integers(1, 3 << 20, 200)])
    for chunk in (64 << 10, 1 << 20, 4 << 20):
        items = batch.plan(lens, chunk)
        seen = {}
        split_phase = True
        last_whole = None
        for doc, lo, hi in items:
            assert lo < hi
            if lens[doc] > chunk:
                assert split_phase, "a large document's tile after a whole document"
                assert hi == lo + 1
            else:
                split_phase = False
                assert (lo, hi) == (0, (lens[doc] + TILE - 1) // TILE)
                if last_whole is not None:
                    assert lens[doc] <= last_whole
                last_whole = lens[doc]
            prev = seen.get(doc, 0)
            assert lo == prev, "tiles of a document out of order"
            seen[doc] = hi
        for d, n in enumerate(lens):
            assert seen.get(d, 0) == (n + TILE - 1) // TILE


def test_mixed_sizes_and_dialects():
    s = batch.mixed_sizes(4096, 6 << 30)
    assert s.min() >= 4 << 10
    assert abs(int(s.sum()) - (6 << 30)) < (6 << 30) // 50
    d = batch.mixed_dialects(4096)
    assert (d == 0).sum() == 2048 and (d == 2).sum() == 1024 and (d == 3).sum() == 1024
