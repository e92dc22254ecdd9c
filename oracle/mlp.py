"""CPU restatement of the entry-region predictor (test infrastructure only:
the product never imports this file).

The predictor has no counterpart in the reference (Mapika/falx guesses a
chunk's entry state without a model, csv_geo.rs:95-149), so this oracle
restates the network's own definition in float64 numpy:

    a1 = b1 + sum_p W1[p*8 + class(byte p)]      h1 = bf16(relu(a1))
    a2 = b2 + h1 @ W2                            h2 = bf16(relu(a2))
    z  = b3 + h2 @ W3                            loss = mean cross-entropy

with every weight used as its bfloat16 rounding, and the backward pass of
that function (gradients with respect to the rounded weights, applied to the
FP32 master copy). `rounding=False` drops every bf16 rounding; the tests pin
this oracle by finite differences in that mode.
"""

import numpy as np

POS, CLS, HID, OUT = 256, 8, 256, 3
OFF_W1 = 0
OFF_B1 = OFF_W1 + POS * CLS * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID * OUT
PARAMS = OFF_B3 + OUT


def byte_class(c):
    """'"' '#' '\\n' ',' '\\r' digit letter other -> 0..7."""
    if c == 0x22:
        return 0
    if c == 0x23:
        return 1
    if c == 0x0A:
        return 2
    if c == 0x2C:
        return 3
    if c == 0x0D:
        return 4
    if 0x30 <= c <= 0x39:
        return 5
    if 0x61 <= (c | 0x20) <= 0x7A:
        return 6
    return 7


def classes(data, starts):
    """Classes of the 256 bytes from each start; outside the data: 7."""
    buf = np.frombuffer(bytes(data), dtype=np.uint8)
    table = np.array([byte_class(c) for c in range(256)], dtype=np.uint8)
    out = np.full((len(starts), POS), 7, dtype=np.uint8)
    for i, s in enumerate(starts):
        lo, hi = max(s, 0), min(s + POS, buf.size)
        if hi > lo:
            out[i, lo - s: hi - s] = table[buf[lo:hi]]
    return out


def bf16(x):
    """Round to the nearest bfloat16 (ties to even); returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w, rounding=True):
    w = np.asarray(w, dtype=np.float64)
    rnd = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    return {
        "W1": rnd(w[OFF_W1:OFF_B1]).reshape(POS * CLS, HID), "b1": w[OFF_B1:OFF_W2],
        "W2": rnd(w[OFF_W2:OFF_B2]).reshape(HID, HID), "b2": w[OFF_B2:OFF_W3],
        "W3": rnd(w[OFF_W3:OFF_B3]).reshape(HID, OUT), "b3": w[OFF_B3:PARAMS],
    }


def forward(w, cls, rounding=True):
    """Activations of every layer for classes cls [n, 256]."""
    P = unpack(w, rounding)
    rnd = bf16 if rounding else (lambda a: a)
    idx = np.arange(POS)[None, :] * CLS + cls.astype(np.int64)
    a1 = P["b1"] + P["W1"][idx].sum(axis=1)
    h1 = rnd(np.maximum(a1, 0.0))
    a2 = P["b2"] + h1 @ P["W2"]
    h2 = rnd(np.maximum(a2, 0.0))
    z = P["b3"] + h2 @ P["W3"]
    return {"P": P, "idx": idx, "a1": a1, "h1": h1, "a2": a2, "h2": h2, "z": z}


def loss(w, cls, labels, rounding=True):
    z = forward(w, cls, rounding)["z"]
    z = z - z.max(axis=1, keepdims=True)
    logp = z - np.log(np.exp(z).sum(axis=1, keepdims=True))
    return float(-logp[np.arange(len(labels)), labels].mean())


def grad(w, cls, labels, rounding=True):
    """(flat gradient of the mean cross-entropy, loss)."""
    f = forward(w, cls, rounding)
    P, n = f["P"], cls.shape[0]
    z = f["z"] - f["z"].max(axis=1, keepdims=True)
    e = np.exp(z)
    p = e / e.sum(axis=1, keepdims=True)
    y = np.zeros_like(p)
    y[np.arange(n), labels] = 1.0
    lval = float(-np.log(p[np.arange(n), labels]).mean())
    dz = (p - y) / n
    g = np.zeros(PARAMS)
    g[OFF_W3:OFF_B3] = (f["h2"].T @ dz).ravel()
    g[OFF_B3:PARAMS] = dz.sum(axis=0)
    d2 = (dz @ P["W3"].T) * (f["a2"] > 0)
    g[OFF_W2:OFF_B2] = (f["h1"].T @ d2).ravel()
    g[OFF_B2:OFF_W3] = d2.sum(axis=0)
    d1 = (d2 @ P["W2"].T) * (f["a1"] > 0)
    gw1 = np.zeros((POS * CLS, HID))
    for pos in range(POS):
        np.add.at(gw1, f["idx"][:, pos], d1)
    g[OFF_W1:OFF_B1] = gw1.ravel()
    g[OFF_B1:OFF_W2] = d1.sum(axis=0)
    return g, lval
