"""Learned initial guess on the GPU: the network's kernels against the CPU
oracle (oracle/cnn_oracle.py), training, and the guess inside the solver.

The convolutions run on the tensor cores with BF16 operands (weights and the
convolution inputs) and FP32 accumulation; the oracle rounds the same values
to BF16 and accumulates in float64.
- Bit-exact pins: with dyadic weights (0, +-1/4), biases and inputs every
  product and partial sum is exact in FP32 whatever the summation order, and
  every activation and back-propagated gradient is exactly representable in
  BF16 (checked on the oracle's values first), so the GPU's forward pass and
  gradient must equal the oracle's bit for bit.
- Random data: a layer's FP32 output can lie on the other side of a BF16
  rounding boundary than the oracle's float64 one, and the next layer then
  sees a value one BF16 step (2^-8 relative) away.  The bar is measured on the
  same data: the oracle is run again with every convolution input moved by up
  to 16 float32 ulps before its BF16 rounding (what another FP32 summation
  order does), and the GPU must stay within 4x the largest such spread.
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


def flip_envelope(fn, ref, seeds=(11, 12, 13, 14, 15)):
    """Largest relative distance from ref of fn(jitter) over a few jitters."""
    return max(rel(fn(np.random.default_rng(s)), ref) for s in seeds)


def dyadic_net(seed, width, depth, cout):
    """A network whose arithmetic is exact: weights in {0, +-1/4} (mostly 0),
    biases in {-1/4, 0, 1/4, 1/2}."""
    net = Cnn(8, width, depth, cout, seed=seed)
    shapes = co.layer_shapes(8, width, depth, cout)
    rng = np.random.default_rng(seed)
    p = np.zeros(net.nparam, np.float32)
    off = 0
    for o, i in shapes:
        nw = o * i * 9
        p[off:off + nw] = rng.choice([-0.25, 0.0, 0.25], size=nw, p=[0.06, 0.88, 0.06])
        p[off + nw:off + nw + o] = rng.choice([-0.25, 0.0, 0.25, 0.5], size=o)
        off += nw + o
    net.set_params(p)
    return net, p, shapes


@pytest.mark.parametrize("shape", [(1, 16, 32), (2, 23, 37)])
def test_tensor_core_forward_bit_exact(shape):
    b, h, w = shape
    net, p, shapes = dyadic_net(21, 32, 3, 4)
    x = np.random.default_rng(2).choice([-1.0, 0.0, 1.0], size=(b, 8, h, w)).astype(np.float32)
    a = co.forward(p, shapes, x)
    assert all(np.array_equal(co.bf16_in(ai), ai) for ai in a[:-1])   # the case is exact
    np.testing.assert_array_equal(net.forward(x), a[-1].astype(np.float32))


def test_tensor_core_gradient_bit_exact():
    """Two layers (the backward-data convolution with the flipped, repacked
    weights, and both weight gradients); 2048 outputs, so the loss gradient
    2 (y - t) / n is exact too."""
    net, p, shapes = dyadic_net(23, 32, 2, 4)
    rng = np.random.default_rng(3)
    x = rng.choice([-1.0, 0.0, 1.0], size=(1, 8, 16, 32)).astype(np.float32)
    t = (rng.integers(-8, 9, size=(1, 4, 16, 32)) / 4.0).astype(np.float32)
    a = co.forward(p, shapes, x)
    gz = 2.0 * (a[-1] - t) / a[-1].size
    assert np.array_equal(co.bf16_in(gz), gz)
    rloss, rg = co.loss_and_grad(p, shapes, x, t)
    assert np.array_equal(rg.astype(np.float32).astype(np.float64), rg)
    loss, g = net.gradient(x, t)
    assert abs(loss - rloss) <= 1e-12 * rloss
    np.testing.assert_array_equal(g, rg.astype(np.float32))


@pytest.mark.parametrize("shape", [(2, 37, 45), (1, 16, 16), (3, 5, 70)])
def test_forward_matches_oracle(shape):
    b, h, w = shape
    net, p, shapes = random_net(5)
    x = np.random.default_rng(1).standard_normal((b, 8, h, w)).astype(np.float32)
    y = net.forward(x)
    ref = co.forward(p, shapes, x)[-1]
    env = flip_envelope(lambda j: co.forward(p, shapes, x, jitter=j)[-1], ref)
    assert rel(y.ravel(), ref.ravel()) < 4 * env + 1e-6, (rel(y.ravel(), ref.ravel()), env)


def test_gradient_matches_oracle():
    net, p, shapes = random_net(7)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((2, 8, 23, 34)).astype(np.float32)
    t = rng.standard_normal((2, 3, 23, 34)).astype(np.float32)
    loss, g = net.gradient(x, t)
    rloss, rg = co.loss_and_grad(p, shapes, x, t)
    jit = [co.loss_and_grad(p, shapes, x, t, jitter=np.random.default_rng(s)) for s in (11, 12, 13, 14, 15)]
    assert abs(loss - rloss) / rloss < 4 * max(abs(jl - rloss) / rloss for jl, _ in jit) + 1e-6
    off = 0
    for o, i in shapes:
        n = o * i * 9 + o
        env = max(rel(jg[off:off + n], rg[off:off + n]) for _, jg in jit)
        e = rel(g[off:off + n], rg[off:off + n])
        assert e < 4 * env + 1e-6, (off, e, env)
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
    judged on every step, and the gain or loss in solver iterations against
    the extrapolated start (the configuration's warm_start=3, which the network
    corrects) is stated and bounded: the network's guess is kept only on steps
    where its FP64 residual is below the extrapolation's, so it may not cost
    more than a few iterations per step."""
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
    assert used[:2] == [-1, -1] and all(u in (0, 1) for u in used[2:5])
    # the network is judged on every step unless 3 judged steps in a row did not
    # pay (it lost the residual test, or won it and took more inner iterations
    # than the last step solved from the previous solution), which switches it
    # off for 16 steps (mclg_ctx.cu guess_bookkeeping)
    run, off, prev = 0, 0, None
    for k, r in enumerate(ev["learned"]["rows"]):
        u = r["used"]
        if k >= 2:
            assert (u == -1) if off > 0 else (u in (0, 1)), (k, used)
        if u == 1:
            run = run + 1 if prev is not None and r["inner"] > prev else 0
        else:
            run += u == 0
            prev = r["inner"]
            off = max(off - 1, 0)
        if run >= 3:
            run, off = 0, 16
    # the extrapolated start (the base of the learned guess) beats the last solution
    assert s["base"]["inner"] < s["previous"]["inner"], s
    gain = s["base"]["inner"] - s["learned"]["inner"]
    print(f"learned guess: {s['learned']['inner']} solver iterations over {s['learned']['steps']} steps against "
          f"{s['base']['inner']} from the extrapolated start ({gain:+d}, {100.0 * gain / s['base']['inner']:+.1f} %); "
          f"the network kept on {s['learned']['used_learned']} steps; validation loss {vloss:.3e} against "
          f"{vzero:.3e} for no correction")
    assert s["learned"]["inner"] <= s["base"]["inner"] + 3 * s["learned"]["steps"], s
