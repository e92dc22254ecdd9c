"""The entry-region predictor's CPU oracle, pinned by finite differences
(float64, no bf16 rounding), plus its byte classes."""

import numpy as np

from oracle import mlp


def small_model(seed):
    rng = np.random.default_rng(seed)
    w = np.zeros(mlp.PARAMS)
    w[mlp.OFF_W1:mlp.OFF_B1] = rng.uniform(-0.15, 0.15, mlp.OFF_B1 - mlp.OFF_W1)
    w[mlp.OFF_B1:mlp.OFF_W2] = rng.uniform(-0.1, 0.1, mlp.HID)
    w[mlp.OFF_W2:mlp.OFF_B2] = rng.uniform(-0.15, 0.15, mlp.HID * mlp.HID)
    w[mlp.OFF_B2:mlp.OFF_W3] = rng.uniform(-0.1, 0.1, mlp.HID)
    w[mlp.OFF_W3:mlp.OFF_B3] = rng.uniform(-0.15, 0.15, mlp.HID * mlp.OUT)
    w[mlp.OFF_B3:mlp.PARAMS] = rng.uniform(-0.1, 0.1, mlp.OUT)
    return w


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(7)
    w = small_model(3)
    cls = rng.integers(0, 8, size=(12, mlp.POS), dtype=np.uint8)
    labels = rng.integers(0, 3, size=12)
    g, _ = mlp.grad(w, cls, labels, rounding=False)
    used_w1 = mlp.OFF_W1 + (np.arange(mlp.POS) * 8 + cls[0]) * mlp.HID  # rows sample 0 touches
    picks = list(used_w1[[0, 50, 255]] + 17) + [mlp.OFF_B1 + 3, mlp.OFF_W2 + 1234, mlp.OFF_B2 + 200,
                                                  mlp.OFF_W3 + 77, mlp.OFF_B3 + 2]
    h = 1e-6
    for i in picks:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (mlp.loss(wp, cls, labels, rounding=False) - mlp.loss(wm, cls, labels, rounding=False)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.01171875, -3.14159, 0.0], dtype=np.float32)
    r = mlp.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: rounds to the even mantissa (1.0)
    assert r[0] == 1.0 and r[1] == 1.0
    assert r[2] == 1.0078125 and r[3] == 1.015625
    assert abs(r[4] + 3.140625) < 1e-12 and r[5] == 0.0


def test_byte_classes():
    cls = mlp.classes(b'"#\n,\r7aZ~', [0, -2, 5])
    assert list(cls[0, :10]) == [0, 1, 2, 3, 4, 5, 6, 6, 7, 7]
    assert list(cls[1, :4]) == [7, 7, 0, 1]
    assert list(cls[2, :5]) == [5, 6, 6, 7, 7]
