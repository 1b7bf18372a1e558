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

The members of amr_configs() also get 0-2 levels of |grad T| refinement of
their base grid (seeded), as the configuration asks; they start from tanh
boundary layers with seeded modes, so the refinement follows the layers.  The
batched solver is the structured multigrid one, so refined members are solved
by the refined-mesh solver, one launch each, after the batched launch.
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


def shard(n, rank=0, world=1):
    """The members rank `rank` of `world` steps: rank, rank + world, ...  Members
    are independent, so the ranks share no data while stepping; the reference
    distributes one model's elements over MPI ranks instead (Parallel.c:167-309),
    which a single device makes unnecessary."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return list(range(rank, n, world))


def configs(n=256, seed=4, sizes=SIZES, members=None):
    ps = draw(n, seed, sizes)
    idx = range(n) if members is None else members
    return [member_config(*ps[i]) for i in idx]


def make(n=256, seed=4, sizes=SIZES, members=None):
    """The ensemble of members `members` (all n by default) of the n drawn."""
    e = Ensemble(configs(n, seed, sizes, members))
    e.initial_temperature()
    return e


def amr_levels(n=256, seed=4):
    """0, 1 or 2 refinement levels per member (seeded)."""
    return np.random.default_rng(seed + 7919).integers(0, 3, n).astype(np.int32)


def amr_configs(n=256, seed=4, sizes=SIZES, members=None):
    """Members with the boundary-layer start that |grad T| refinement follows."""
    out = configs(n, seed, sizes, members)
    for c in out:
        c.ic_kind = 2
        c.ic_bl_thickness = 0.02
        c.ic_modes = 8
        c.ic_mode_amp = 0.005
    return out


def make_amr(n=256, seed=4, sizes=SIZES, members=None):
    lv = amr_levels(n, seed)
    if members is not None:
        lv = np.ascontiguousarray(lv[list(members)])
    e = Ensemble(amr_configs(n, seed, sizes, members), lv)
    e.initial_temperature()
    return e
