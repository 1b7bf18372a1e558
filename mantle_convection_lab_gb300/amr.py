"""Configuration 2: |grad T| adaptive refinement with periodic remeshing.

    with AmrRun() as run:           # configs/cfg2_amr_128.input
        for _ in range(200):
            st = run.step()         # remeshes before every 10th step

The model starts on the uniform 128 x 128 base grid (leaf level 7 of the
1024 x 1024 finest grid).  Before step 0 and every `remesh_every` steps the
device flags elements with |grad T| > frac * max, the host builds the new
2:1-balanced tree (flagged regions at level base + extra) and the model is
rebuilt on it in place with T carried over (mclg_amr_remesh).
"""
import os
import time

import numpy as np

from .api import Config, Model

HERE = os.path.dirname(os.path.abspath(__file__))
CFG2_INPUT = os.path.join(HERE, "configs", "cfg2_amr_128.input")


def uniform_leaves(finest_level, base_level):
    """Leaf start codes of the uniform grid at base_level inside finest_level."""
    return np.arange(0, 1 << (2 * finest_level), 1 << (2 * (finest_level - base_level)), dtype=np.int32)


class AmrRun:
    """Configuration 2's run: remesh every `remesh_every` steps.  With lag > 0 a
    remesh after the first is asynchronous: its flags come from the temperature
    at step k, its mesh is built on a host thread while steps k .. k+lag-1 run
    on the old mesh, and it is swapped in before step k+lag (the fields carried
    over are those of that moment)."""

    def __init__(self, config=None, base_level=7, extra_levels=3, frac=0.2, remesh_every=10, lag=0):
        self.config = config if config is not None else Config.from_input(CFG2_INPUT)
        self.F = self.config.level - 1
        self.base, self.target = base_level, min(base_level + extra_levels, self.F)
        self.frac, self.every, self.lag = frac, remesh_every, lag
        self.model = Model(self.config, leaves=uniform_leaves(self.F, self.base))
        self.model.initial_temperature()
        self.steps = 0
        self.remeshes = 0
        self._pending = False
        self.ms_begin, self.ms_end = [], []    # host wall time of each remesh_begin / remesh_end

    def remesh(self):
        n = self.model.remesh(self.frac, self.base, self.target)
        self.remeshes += 1
        return n

    def step(self):
        k = self.steps % self.every
        if self._pending and k == self.lag:
            t0 = time.perf_counter()
            self.model.remesh_end()
            self.ms_end.append(1e3 * (time.perf_counter() - t0))
            self._pending = False
            self.remeshes += 1
        if k == 0:
            if self.lag > 0 and self.steps > 0:
                t0 = time.perf_counter()
                self.model.remesh_begin(self.frac, self.base, self.target)
                self.ms_begin.append(1e3 * (time.perf_counter() - t0))
                self._pending = True
            else:
                self.remesh()
        st = self.model.step()
        self.steps += 1
        return st

    def close(self):
        self.model.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
