"""Learned speculation on the GPU: the predictor's forward and backward
kernels against the CPU oracle, and the speculative index against the plain
one under every kind of prediction (constant, model, random, all wrong)."""

import numpy as np
import pytest

import falx_gb300 as fx
from conftest import DIALECT_ALPHABETS, Rng, random_doc
from falx_gb300 import gen, speculation
from oracle import mlp

pytestmark = pytest.mark.gpu

NSTATES = {fx.CSV: 2, fx.CSV_HASH: 3, fx.TSV: 1, fx.LOGFMT: 4, fx.NDJSON: 4}


def rel_err(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_forward_matches_oracle(engine):
    import torch

    model = engine.model_create(seed=11)
    w = model.get()
    rng = np.random.default_rng(5)
    cls = rng.integers(0, 8, size=(40, mlp.POS), dtype=np.uint8)
    z, pred = model.forward(torch.from_numpy(cls).cuda())
    want = mlp.forward(w, cls)["z"]
    # FP32 accumulation against float64; bf16 re-rounding of a hidden unit
    # near a rounding boundary moves a logit by at most a few bf16 ulps.
    assert rel_err(z.cpu().numpy(), want) < 2e-3
    assert np.abs(z.cpu().numpy() - want).max() < 5e-2
    zz = z.cpu().numpy()
    assert np.array_equal(pred.cpu().numpy(), zz.argmax(axis=1))
    model.close()


def test_gradient_matches_oracle(engine):
    import torch

    model = engine.model_create(seed=12)
    w = model.get()
    rng = np.random.default_rng(6)
    cls = rng.integers(0, 8, size=(48, mlp.POS), dtype=np.uint8)
    # skew classes like text: mostly letters and digits
    cls[rng.random(cls.shape) < 0.6] = 6
    labels = rng.integers(0, 3, size=48).astype(np.uint8)
    g, loss = model.grad(torch.from_numpy(cls).cuda(), torch.from_numpy(labels).cuda())
    want, wl = mlp.grad(w, cls, labels.astype(np.int64))
    g = g.cpu().numpy().astype(np.float64)
    assert abs(loss - wl) <= 1e-4 * abs(wl)
    for lo, hi in [(mlp.OFF_W1, mlp.OFF_B1), (mlp.OFF_B1, mlp.OFF_W2), (mlp.OFF_W2, mlp.OFF_B2),
                   (mlp.OFF_B2, mlp.OFF_W3), (mlp.OFF_W3, mlp.OFF_B3), (mlp.OFF_B3, mlp.PARAMS)]:
        assert rel_err(g[lo:hi], want[lo:hi]) < 1e-2, (lo, hi)
    model.close()


def test_byte_classes_match_oracle(engine):
    import torch

    doc = gen.generate(gen.ADVERSARIAL, 1 << 20)
    starts = np.array([0, 5, 1000, len(doc) - 100, len(doc) - 1, -50], dtype=np.int64)
    got = engine.byte_classes(doc, torch.from_numpy(starts)).cpu().numpy()
    assert np.array_equal(got, mlp.classes(doc.tobytes(), starts))


def truth_states(engine, doc, dialect):
    import torch

    d = torch.from_numpy(np.frombuffer(bytes(doc), dtype=np.uint8).copy()).cuda()
    return d, speculation.tile_entry_states(engine, d, dialect).cpu().numpy()


def check_speculative(engine, doc, dialect, assumed_fn):
    import torch

    d, truth = truth_states(engine, doc, dialect)
    want = engine.index_structurals(d, dialect).cpu().numpy()
    assumed = assumed_fn(truth)
    got, tiles, wrong = engine.index_structurals_speculative(d, dialect, assumed=torch.from_numpy(assumed).cuda())
    assert np.array_equal(got.cpu().numpy(), want)
    assert tiles == truth.size
    a = assumed.astype(np.int64)
    hedged = a == 0xFF
    a[(a >= NSTATES[dialect]) & ~hedged] = 0
    assert wrong == int(((a[1:] != truth[1:]) & ~hedged[1:]).sum())
    return wrong


@pytest.mark.parametrize("dialect", [fx.CSV, fx.CSV_HASH, fx.LOGFMT, fx.NDJSON, fx.TSV])
def test_speculative_index_any_assumption(engine, dialect):
    kind = {fx.CSV: gen.CSV_GEO, fx.CSV_HASH: gen.ADVERSARIAL, fx.LOGFMT: gen.LOGFMT, fx.NDJSON: gen.NDJSON,
            fx.TSV: gen.TSV}[dialect]
    doc = gen.generate(kind, 12 << 20)
    ns = NSTATES[dialect]
    rng = np.random.default_rng(dialect)
    check_speculative(engine, doc, dialect, lambda t: np.zeros_like(t))
    check_speculative(engine, doc, dialect, lambda t: t.copy())
    check_speculative(engine, doc, dialect, lambda t: rng.integers(0, ns, size=t.size).astype(np.uint8))
    # a mix of guesses, no-guess tiles (0xFF) and out-of-range values
    check_speculative(engine, doc, dialect,
                      lambda t: rng.choice(np.array([0, 1, 2, 3, 0xFF, 7], dtype=np.uint8), size=t.size))
    wrong = check_speculative(engine, doc, dialect, lambda t: ((t.astype(np.int64) + 1) % max(ns, 2)).astype(np.uint8))
    if ns > 1:
        assert wrong == t_size(doc) - 1


def t_size(doc):
    return (len(doc) + fx._lib.SPEC_TILE - 1) // fx._lib.SPEC_TILE


def test_speculative_index_random_docs(engine):
    import torch

    rng = Rng(0x5BEC)
    for dialect in (fx.CSV, fx.CSV_HASH, fx.LOGFMT, fx.NDJSON):
        doc = random_doc(rng, DIALECT_ALPHABETS[dialect], 300_000)
        nrng = np.random.default_rng(dialect + 10)
        check_speculative(engine, doc, dialect,
                          lambda t: nrng.integers(0, NSTATES[dialect], size=t.size).astype(np.uint8))
    # small and empty inputs
    for doc in (b"", b"a", b'"\n' * 40_000, b"#x\n" * 30_000):
        want = engine.index_structurals(doc, fx.CSV_HASH).cpu().numpy() if doc else np.zeros(0, np.uint32)
        got, _, _ = engine.index_structurals_speculative(doc if doc else b"", fx.CSV_HASH,
                                                         assumed=torch.full((8,), 1, dtype=torch.uint8))
        assert np.array_equal(got.cpu().numpy(), want)


def test_trained_model_beats_constant_guess(engine):
    # Train on separately seeded documents, evaluate on another seed: the
    # network must mispredict fewer tiles than the constant guess, and the
    # speculative index stays identical to the plain one.
    model, info = speculation.train_model(engine, train_bytes=96 << 20, epochs=3, stride=512)
    assert info["final_loss"] < 1.0
    doc = gen.generate(gen.ADVERSARIAL, 64 << 20, seed=speculation.EVAL_SEED)
    m = speculation.misprediction(engine, model, doc)
    assert m["constant_wrong"] > 0
    assert m["model_wrong"] < m["constant_wrong"], (m, info)
    got, tiles, wrong = engine.index_structurals_speculative(doc, fx.CSV_HASH, model=model)
    want = engine.index_structurals(doc, fx.CSV_HASH)
    assert np.array_equal(got.cpu().numpy(), want.cpu().numpy())
    assert wrong == m["model_wrong"]
    # hedging the uncertain tiles only removes mispredictions
    model.set_confidence(0.9)
    got, _, wrong_h = engine.index_structurals_speculative(doc, fx.CSV_HASH, model=model)
    assert np.array_equal(got.cpu().numpy(), want.cpu().numpy())
    assert wrong_h <= wrong
    model.close()
