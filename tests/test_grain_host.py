"""Grain-size rheology on the host (csrc/host/mclg_grain.c), the engine's
implementation of Grain_size_evolution.c:3-152, against the reference's own
runs on single-level meshes (tests/golden/gd_l5: cold top, the grain size stays
at 1e-3 and the clip sets the viscosity near the top; gdw_l5: a warmer top, the
grain size evolves and the clip acts at both ends).  Each call gets the
reference's inputs of that step (its temperature after the previous step, its
stress of the previous step, its model time) and must leave the reference's
grain size and viscosity, bit for bit where the routine wrote them."""
import numpy as np
import pytest
from conftest import golden, golden_input

from mantle_convection_lab_gb300 import Config, GrainSize, Mesh


@pytest.mark.parametrize("case,threads", [("gd_l5", 1), ("gdw_l5", 4)])
def test_grain_size_matches_reference(case, threads):
    g = golden(case)
    c = Config.from_input(golden_input(case))
    m = Mesh(c)
    X = m.get("X")
    nno = X.size // 2
    z = X[nno:]
    shallow = 2890 * (1.0 - z) <= 200.0
    gs = GrainSize()
    steps = g["series/steps"]
    for s in steps:
        T = m.initial_temperature() if s == 0 else g[f"heat{s - 1:04d}/T"]
        vis0 = np.exp(c.A * (c.refT - T)) * np.where(z < 0.77, c.lower_mantle_jump, 1.0)
        stress = np.zeros(nno) if s == 0 else g[f"step{s - 1:04d}/stress"]
        model_time = 0.0 if s == 0 else g["series/model_time"][s - 1]
        _, vis = gs.update(X, T, stress, vis0, model_time, c.Rayleigh, c.lowest_vis, c.highest_vis, threads)
        want_vis = g[f"step{s:04d}/vis"]
        np.testing.assert_array_equal(gs.grain_size(), g[f"step{s:04d}/gs"])
        if s > 0:
            np.testing.assert_array_equal(vis[shallow], want_vis[shallow])
        np.testing.assert_allclose(vis[~shallow], want_vis[~shallow], rtol=1e-15, atol=0)
    gs.close()


def test_first_call_only_initialises():
    gs = GrainSize()
    X = np.array([0.0, 1.0, 0.99, 0.5])   # two nodes: z = 0.99 (shallow), 0.5 (deep)
    stress, vis = gs.update(X, np.array([0.1, 0.5]), np.array([3.0, 4.0]), np.array([1.0, 2.0]), 1.0, 1e5, 1e-3,
                            1e3)
    np.testing.assert_array_equal(gs.grain_size(), [1e-3, 1e-3])
    np.testing.assert_array_equal(stress, [3.0, 4.0])
    np.testing.assert_array_equal(vis, [1.0, 2.0])
    gs.close()
