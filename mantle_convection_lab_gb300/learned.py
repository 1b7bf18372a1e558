"""Learned initial guess: training data, training and evaluation.

Training samples are snapshots that the solver itself produces: with the
guess in GUESS_RECORD mode every solve (after the first two) leaves the
features it would feed the network -- T, 0.2 log10 eta and the last two
solutions on the coarse node grid -- and the target, the change from the last
solution to the converged one.  The network is trained on the device by the
library's kernels (mclg_cnn_train) and saved with mclg_cnn_save.

    python -m mantle_convection_lab_gb300.learned train --out guess.bin \\
        --input mantle_convection_lab_gb300/configs/cfg3_mg_1024.input --level 9 --seeds 1,2,3 --steps 120
    python -m mantle_convection_lab_gb300.learned eval --net guess.bin --steps 30
"""
import argparse
import json
import os
import sys
import time

import numpy as np

from .api import GUESS_FORCED, GUESS_LEARNED, GUESS_OFF, GUESS_RECORD, Cnn, Config, MclgError, Model

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_INPUT = os.path.join(HERE, "configs", "cfg3_mg_1024.input")
DEFAULT_NET = os.path.join(HERE, "weights", "guess_cfg3.bin")


def make_config(path, level=None, seed=None, **over):
    c = Config.from_input(path)
    if level is not None:
        c.level = level
    if seed is not None:
        c.ic_seed = seed
    for k, v in over.items():
        setattr(c, k, v)
    return c


def generate(path=DEFAULT_INPUT, seeds=(1,), steps=100, grid=128, level=None, skip=0, every=1, **over):
    """Run one model per seed for `steps` steps in GUESS_RECORD mode and stack
    the samples (features [n, 8, g+1, g+1], targets [n, 3, g+1, g+1]).  The
    target is relative to the configuration's warm_start guess."""
    xs, ys = [], []
    for seed in seeds:
        with Model(make_config(path, level, seed, **over)) as m:
            m.initial_temperature()
            m.guess_set(GUESS_RECORD, grid)
            for s in range(steps):
                m.step()
                if s < skip or (s - skip) % every:
                    continue
                try:
                    x, y = m.guess_sample()
                except MclgError:
                    continue
                xs.append(x)
                ys.append(y)
    return np.stack(xs), np.stack(ys)


def train(X, Y, width=32, depth=6, iters=2000, batch=16, lr=1e-3, seed=0, val_frac=0.1):
    """Fit a network on (X, Y); returns (net, loss trace, validation loss,
    validation loss of the zero prediction = keeping the last solution)."""
    n = X.shape[0]
    nval = max(1, int(round(n * val_frac))) if n > 1 else 0
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n)
    val, tr = perm[:nval], perm[nval:] if n > 1 else perm
    net = Cnn(X.shape[1], width, depth, Y.shape[1], seed=seed)
    trace = net.train(X[tr], Y[tr], batch=min(batch, len(tr)), iters=iters, lr=lr, seed=seed)
    vloss = vzero = float("nan")
    if nval:
        pred = np.concatenate([net.forward(X[val[i:i + 8]]) for i in range(0, nval, 8)])
        vloss = float(np.mean((pred - Y[val]) ** 2))
        vzero = float(np.mean(Y[val] ** 2))
    return net, trace, vloss, vzero


def evaluate(net, path=DEFAULT_INPUT, steps=30, grid=128, level=None, seed=None, extra=(), **over):
    """The same run without ("base") and with the network ("learned"): per-step
    inner iterations, which guess the solver kept, and time per step.  Both
    start each step from the configuration's warm_start guess, which the
    network corrects.  `extra` adds runs: "forced" takes the network's guess
    on every step without judging it, "previous" and "extrapolate" use
    warm_start=1 (last solution) and 3 (extrapolation) without a network."""
    out = {}
    base = make_config(path, level, seed, **over).warm_start
    runs = [("base", GUESS_OFF, base), ("learned", GUESS_LEARNED, base)]
    runs += [{"forced": ("forced", GUESS_FORCED, base), "previous": ("previous", GUESS_OFF, 1),
              "extrapolate": ("extrapolate", GUESS_OFF, 3)}[k] for k in extra]
    for label, mode, warm in runs:
        with Model(make_config(path, level, seed, **dict(over, warm_start=warm))) as m:
            m.initial_temperature()
            if mode != GUESS_OFF:
                m.guess_set(mode, grid, net)
            rows = []
            for _ in range(steps):
                st = m.step()
                rows.append({"inner": st.cg_cycles, "outer": st.uzawa_cycles, "refine": st.refine_passes,
                             "ms": st.ms_total, "ms_guess": st.ms_guess, "used": st.guess_used,
                             "res_learned": st.res_guess_learned, "res_prev": st.res_guess_prev,
                             "res": max(st.res_momentum, st.res_continuity)})
            out[label] = {"rows": rows, "T": m.get("T"), "V0": m.get("V0"), "P": m.get("P")}
    return out


def summary(ev, skip=2):
    """Totals over the steps after the first `skip` (the network needs two
    earlier solutions)."""
    s = {}
    for k, v in ev.items():
        r = v["rows"][skip:]
        s[k] = {"steps": len(r), "inner": int(sum(x["inner"] for x in r)), "outer": int(sum(x["outer"] for x in r)),
                "ms": float(sum(x["ms"] for x in r)), "used_learned": int(sum(1 for x in r if x["used"] == 1)),
                "max_res": float(max(x["res"] for x in r)) if r else 0.0}
    return s


def main(argv=None):
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--input", default=DEFAULT_INPUT)
    t.add_argument("--level", type=int, default=None)
    t.add_argument("--seeds", default="1,2,3")
    t.add_argument("--steps", type=int, default=120)
    t.add_argument("--grid", type=int, default=128)
    t.add_argument("--iters", type=int, default=3000)
    t.add_argument("--batch", type=int, default=16)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--width", type=int, default=32)
    t.add_argument("--depth", type=int, default=6)
    t.add_argument("--out", default=DEFAULT_NET)
    e = sub.add_parser("eval")
    e.add_argument("--input", default=DEFAULT_INPUT)
    e.add_argument("--level", type=int, default=None)
    e.add_argument("--seed", type=int, default=None)
    e.add_argument("--steps", type=int, default=30)
    e.add_argument("--grid", type=int, default=128)
    e.add_argument("--net", default=DEFAULT_NET)
    a = ap.parse_args(argv)
    if a.cmd == "train":
        t0 = time.perf_counter()
        X, Y = generate(a.input, [int(s) for s in a.seeds.split(",")], a.steps, a.grid, a.level)
        t1 = time.perf_counter()
        net, trace, vloss, vzero = train(X, Y, a.width, a.depth, a.iters, a.batch, a.lr)
        t2 = time.perf_counter()
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        net.save(a.out)
        print(json.dumps({"samples": int(X.shape[0]), "grid": a.grid, "params": net.nparam,
                          "generate_s": t1 - t0, "train_s": t2 - t1, "loss_first": float(trace[0]),
                          "loss_last": float(np.mean(trace[-50:])), "val_loss": vloss, "val_loss_zero": vzero,
                          "out": a.out}))
    else:
        net = Cnn.load(a.net)
        ev = evaluate(net, a.input, a.steps, a.grid, a.level, a.seed)
        print(json.dumps({"summary": summary(ev),
                          "per_step": {k: [(r["inner"], r["used"]) for r in v["rows"]] for k, v in ev.items()}}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
