"""The CPU oracle of the learned-guess network, pinned by finite differences.

The reference has no learned component, so the oracle (oracle/cnn_oracle.py)
is pinned against calculus instead: its back-propagated gradient must match
central differences of its own loss in float64 (without weight rounding),
and its bfloat16 rounding must match the bit-level definition.
"""
import numpy as np

import cnn_oracle as co


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2**-8, 1.0 + 2**-7 + 2**-8, 1.0 + 2**-7 + 2**-8 + 2**-10, -3.14159, 65504.0, 1e-30],
                 np.float32)
    r = co.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0                  # tie to even (down)
    assert r[2] == np.float32(1.0 + 2**-6)              # tie to even (up)
    assert r[3] == np.float32(1.0 + 2**-6)              # above the tie rounds up
    assert (r.view(np.uint32) & 0xFFFF).max() == 0
    assert np.all(np.abs(r - x) <= np.abs(x) * 2**-8)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    shapes = co.layer_shapes(3, 4, 3, 2)
    n = sum(o * i * 9 + o for o, i in shapes)
    p = rng.standard_normal(n) * 0.4
    x = rng.standard_normal((2, 3, 5, 6))
    t = rng.standard_normal((2, 2, 5, 6))

    def loss(q):
        layers = co.unpack(q, shapes)
        a = x
        for l, (W, b) in enumerate(layers):
            z = co.conv(a, W, b)
            a = np.maximum(z, 0) if l + 1 < len(layers) else z
        return np.mean((a - t) ** 2)

    # float64 path of the oracle (no rounding)
    L, g = co.loss_and_grad(p.astype(np.float32).astype(np.float64), shapes, x, t, quantize=False)
    p32 = p.astype(np.float32).astype(np.float64)
    assert abs(L - loss(p32)) < 1e-12
    h = 1e-6
    idx = rng.choice(n, 40, replace=False)
    fd = np.array([(loss(p32 + h * np.eye(1, n, i)[0]) - loss(p32 - h * np.eye(1, n, i)[0])) / (2 * h) for i in idx])
    assert np.linalg.norm(fd - g[idx]) / np.linalg.norm(fd) < 1e-6


def test_adam_matches_definition():
    w = np.array([0.5, -1.0], np.float32)
    g = np.array([0.1, -0.2], np.float32)
    w1, m1, v1 = co.adam(w, g, np.zeros(2), np.zeros(2), 1, lr=0.01)
    # first step of Adam moves every weight by lr * sign(g) (up to eps)
    assert np.allclose(w1, w - 0.01 * np.sign(g), atol=1e-6)
