"""Learned speculation for the csv_hash structural index.

The entry-region predictor is trained only on labels produced by the exact
scan over generated documents: for a start offset every `stride` bytes of a
training document, the input is the classes of the 256 bytes from there and
the label is the exact region state (NORMAL / QUOTE / COMMENT) before that
byte (falx_region_states). Training documents use seeds distinct from the
measured ones. Everything here runs on the engine's own kernels.
"""

import time

from . import gen
from ._lib import CSV_HASH, SPEC_TILE

# Training documents: same generator as the measured adversarial workload,
# separately seeded.
TRAIN_SEED = 0x7EA1_5EED_0000_0001
EVAL_SEED = 0x7EA1_5EED_0000_0002


def training_set(engine, docs, dialect=CSV_HASH, stride=1024):
    """(classes [n, 256] uint8, labels [n] uint8) on the device."""
    torch = engine.torch
    cls_parts, lab_parts = [], []
    for doc in docs:
        d = engine.to_device(doc)
        if d.data_ptr() % 16:
            d = d.clone()  # block k of the labels is file position 64k for 16-byte aligned data
        states = engine.region_states(d, dialect)
        starts = torch.arange(0, d.numel(), stride, device=d.device, dtype=torch.int64)
        lab_parts.append(states[starts // 64].contiguous())
        cls_parts.append(engine.byte_classes(d, starts))
    return torch.cat(cls_parts), torch.cat(lab_parts)


def tile_entry_states(engine, data, dialect=CSV_HASH):
    """Exact entry state of every speculation tile of 16-byte aligned `data`."""
    states = engine.region_states(data, dialect)
    return states[:: SPEC_TILE // 64].contiguous()


def train_model(engine, train_bytes=256 << 20, epochs=2, batch=512, lr=1e-3, seed=1, stride=1024,
                doc_seed=TRAIN_SEED, kind=gen.ADVERSARIAL, dialect=CSV_HASH):
    """Train a predictor on about `train_bytes` of generated documents.
    Returns (model, info)."""
    torch = engine.torch
    t0 = time.time()
    doc = gen.generate(kind, train_bytes, seed=doc_seed)
    cls, labels = training_set(engine, [doc], dialect, stride)
    g = torch.Generator(device=cls.device)
    g.manual_seed(seed)
    perm = torch.randperm(cls.shape[0], device=cls.device, generator=g)
    cls, labels = cls[perm].contiguous(), labels[perm].contiguous()
    t1 = time.time()
    model = engine.model_create(seed)
    loss = model.train(cls, labels, batch=batch, epochs=epochs, lr=lr)
    torch.cuda.synchronize()
    t2 = time.time()
    counts = torch.bincount(labels.long(), minlength=3).tolist()
    return model, {"samples": int(cls.shape[0]), "label_counts": counts, "epochs": epochs, "batch": batch,
                   "final_loss": loss, "label_s": round(t1 - t0, 3), "train_s": round(t2 - t1, 3)}


def misprediction(engine, model, data, dialect=CSV_HASH):
    """Per-tile misprediction counts of the model and of the constant
    'outside any region' guess against the exact entry states."""
    d = engine.to_device(data)
    if d.data_ptr() % 16:
        d = d.clone()
    truth = tile_entry_states(engine, d, dialect)
    pred = model.predict_tiles(d)
    n = min(truth.numel(), pred.numel())
    truth, pred = truth[1:n], pred[1:n]  # tile 0's entry is known
    return {"tiles": n, "model_wrong": int((truth != pred).sum()), "constant_wrong": int((truth != 0).sum())}


def time_index(engine, fn, reps=5):
    """Best-of-reps device time (ms) of fn() on the current stream."""
    torch = engine.torch
    stream = torch.cuda.current_stream()
    fn()
    torch.cuda.synchronize()
    best = float("inf")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(reps):
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def calibrate_confidence(engine, model, data, dialect=CSV_HASH, candidates=(0.0, 0.8, 0.9, 0.95, 0.98, 0.99)):
    """Pick the hedging threshold with the fastest predict + speculative
    scan on a calibration document (not the measured one)."""
    d = engine.to_device(data)
    best = None
    for conf in candidates:
        model.set_confidence(conf)
        t = time_index(engine, lambda: engine.index_structurals_speculative(d, dialect, model=model), reps=3)
        if best is None or t < best[1]:
            best = (conf, t)
    model.set_confidence(best[0])
    return best[0]
