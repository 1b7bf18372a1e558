"""Configuration 4: a batched ensemble of independent convection models.

Each member is configuration 3's model (free-slip unit box, T = 1 at the bottom
and 0 at the top, seeded initial temperature) with its own mesh size and
parameters drawn from a seeded stream:
- elements per side from {32, 64, 128, 256};
- Rayleigh number log-uniform in [1e5, 1e7];
- viscosity contrast c log-uniform in [1, 1e4], eta = exp(-ln(c) T);
- a seeded conductive profile with a cosine mode and noise of amplitude 1e-3.
All members use the mixed-precision converged solver (FP32 multigrid inside
FP64 refinement, MINRES correction, extrapolated warm start) and are stepped
together by mclg_ensemble_step: one batched solver launch per step.

Members are uniform meshes (no AMR levels): the batched solver is the
structured multigrid one.
"""
import math
import os

import numpy as np

from .api import Config, Ensemble

HERE = os.path.dirname(os.path.abspath(__file__))
BASE_INPUT = os.path.join(HERE, "configs", "cfg3_mg_1024.input")
SIZES = (32, 64, 128, 256)


def member_config(n_side, rayleigh, contrast, seed, base=BASE_INPUT):
    c = Config.from_input(base)
    c.level = int(round(math.log2(n_side))) + 1
    c.mg_min_level = 1
    c.Rayleigh = rayleigh
    c.A = math.log(contrast)
    c.refT = 0.0
    c.vis_min = 1.0 / contrast
    c.vis_max = 1.0
    c.ic_kind = 1
    c.ic_seed = seed
    c.ic_noise = 1e-3
    c.T_mantle_perturb = 0.01
    c.T_wave_number = 1
    c.max_timestep = 99
    return c


def draw(n=256, seed=4, sizes=SIZES):
    """Parameters of n members: (elements per side, Ra, contrast, seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        side = int(sizes[rng.integers(len(sizes))])
        ra = float(10 ** rng.uniform(5, 7))
        contrast = float(10 ** rng.uniform(0, 4))
        out.append((side, ra, contrast, 1000 + i))
    return out


def configs(n=256, seed=4, sizes=SIZES):
    return [member_config(*p) for p in draw(n, seed, sizes)]


def make(n=256, seed=4, sizes=SIZES):
    e = Ensemble(configs(n, seed, sizes))
    e.initial_temperature()
    return e
