"""Learned initial guess on the GPU: the network's kernels against the CPU
oracle (oracle/cnn_oracle.py), training, and the guess inside the solver.

Tolerances: the kernels accumulate in FP32 (the oracle in float64) over at
most 9 x 32 products per output, so forward outputs agree to ~1e-6 relative;
gradients sum over every pixel of the batch in FP32 and are held to 1e-4.
"""
import numpy as np
import pytest
from conftest import golden_input, rel

import cnn_oracle as co
from mantle_convection_lab_gb300 import Cnn, Config, Model
from mantle_convection_lab_gb300.api import GUESS_LEARNED, GUESS_OFF, GUESS_RECORD
from mantle_convection_lab_gb300 import learned

pytestmark = pytest.mark.gpu


def random_net(seed, cin=8, width=32, depth=6, cout=3, scale=0.2):
    net = Cnn(cin, width, depth, cout, seed=seed)
    p = np.random.default_rng(seed).standard_normal(net.nparam).astype(np.float32) * scale
    net.set_params(p)
    return net, p, co.layer_shapes(cin, width, depth, cout)


@pytest.mark.parametrize("shape", [(2, 37, 45), (1, 16, 16), (3, 5, 70)])
def test_forward_matches_oracle(shape):
    b, h, w = shape
    net, p, shapes = random_net(5)
    x = np.random.default_rng(1).standard_normal((b, 8, h, w)).astype(np.float32)
    y = net.forward(x)
    ref = co.forward(p, shapes, x)[-1]
    assert rel(y.ravel(), ref.ravel()) < 1e-5


def test_gradient_matches_oracle():
    net, p, shapes = random_net(7)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((2, 8, 23, 34)).astype(np.float32)
    t = rng.standard_normal((2, 3, 23, 34)).astype(np.float32)
    loss, g = net.gradient(x, t)
    rloss, rg = co.loss_and_grad(p, shapes, x, t)
    assert abs(loss - rloss) / rloss < 1e-6
    off = 0
    for o, i in shapes:
        n = o * i * 9 + o
        assert rel(g[off:off + n], rg[off:off + n]) < 1e-4, (off, rel(g[off:off + n], rg[off:off + n]))
        off += n


def test_adam_matches_oracle():
    net, p, _ = random_net(9)
    rng = np.random.default_rng(4)
    m = np.zeros(net.nparam, np.float32)
    v = np.zeros(net.nparam, np.float32)
    w = p.copy()
    for t in (1, 2, 3):
        g = rng.standard_normal(net.nparam).astype(np.float32)
        net.adam_step(g, 1e-3)
        w, m, v = co.adam(w, g, m, v, t, 1e-3)
    assert rel(net.params(), w) < 1e-6


def test_training_fits_a_teacher_network(tmp_path):
    teacher, _, _ = random_net(11, width=8, depth=2, scale=0.3)
    rng = np.random.default_rng(5)
    X = rng.standard_normal((64, 8, 20, 20)).astype(np.float32)
    Y = teacher.forward(X)
    student = Cnn(8, 16, 3, 3, seed=3)
    trace = student.train(X, Y, batch=8, iters=400, lr=3e-3, seed=1)
    assert np.isfinite(trace).all()
    assert trace[-20:].mean() < 0.1 * trace[:5].mean(), (trace[:5], trace[-20:])
    # save / load keeps the parameters bit for bit
    path = str(tmp_path / "net.bin")
    student.save(path)
    again = Cnn.load(path)
    assert np.array_equal(again.params(), student.params())
    np.testing.assert_array_equal(again.forward(X[:2]), student.forward(X[:2]))


def _small(level=7, **over):
    c = Config.from_input(learned.DEFAULT_INPUT)
    c.level = level
    for k, v in over.items():
        setattr(c, k, v)
    return c


def test_record_mode_samples_and_guess_requires_converged_solver():
    with Model(Config.from_input(golden_input("cfg1_l5"))) as m:
        with pytest.raises(Exception):
            m.guess_set(GUESS_RECORD, 8)      # FP64 replica: no learned guess
    with Model(_small()) as m:
        m.initial_temperature()
        m.guess_set(GUESS_RECORD, 32)
        m.step()
        m.step()
        with pytest.raises(Exception):
            m.guess_sample()                   # needs two earlier solutions
        m.step()
        x, y = m.guess_sample()
        assert x.shape == (8, 33, 33) and y.shape == (3, 33, 33)
        assert np.isfinite(x).all() and np.isfinite(y).all()
        # velocity channels are scaled by the RMS speed of the last solution
        assert abs(np.sqrt(np.mean(x[2] ** 2 + x[3] ** 2)) - 1.0) < 1e-5


def test_learned_guess_in_the_solver():
    """Train on two seeded 64x64 runs, then run a third seed with and without
    the network: both reach the residual, the fields agree, the network is
    judged on every step, and the iteration counts are reported."""
    path = learned.DEFAULT_INPUT
    X, Y = learned.generate(path, seeds=(1, 2), steps=30, grid=32, level=7)
    assert X.shape[0] == 2 * 28
    net, trace, vloss, vzero = learned.train(X, Y, iters=300, batch=8, lr=1e-3)
    assert np.isfinite(trace).all()
    ev = learned.evaluate(net, path, steps=12, grid=32, level=7, seed=3, extra=("previous",))
    s = learned.summary(ev)
    rtol = Config.from_input(path).stokes_rtol
    for k in ("base", "learned", "previous"):
        assert s[k]["max_res"] < rtol, (k, s[k])
    for f in ("T", "V0", "P"):
        assert rel(ev["learned"][f], ev["base"][f]) < 1e-6, f
    used = [r["used"] for r in ev["learned"]["rows"]]
    assert used[:2] == [-1, -1] and all(u in (0, 1) for u in used[2:])
    # the extrapolated start (the base of the learned guess) beats the last solution
    assert s["base"]["inner"] < s["previous"]["inner"], s
    print("learned guess:", s, "val loss", vloss, "vs the base guess", vzero)
