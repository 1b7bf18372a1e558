"""Host mesh and numbering against the reference's own arrays (bit-exact).

Fixtures were dumped from the reference built from source (tests/golden/make_golden.py).
Covers the uniform mesh, boundary-band refinement with hanging nodes (develop_mode 11),
top-band (12), graded multi-band (13) and lower-half (14) refinement, on every MG level.
"""
import numpy as np
import pytest
from conftest import golden, golden_input

from mantle_convection_lab_gb300 import Config, Mesh

CASES = ["cfg1_l5", "hang11_l6", "dev12_l7", "dev13_l8", "dev14_l7", "vc_l6"]
INT_KEYS = ["Mcode", "node", "ien", "id", "heat_id", "lm"]


@pytest.mark.parametrize("case", CASES)
def test_numbering_bit_exact(case):
    g = golden(case)
    m = Mesh(Config.from_input(golden_input(case)))
    levels = sorted({int(k.split("@")[1]) for k in g.files if k.startswith("mesh/Mcode@")})
    assert levels
    for lev in levels:
        for k in INT_KEYS:
            a, b = m.get(k, lev), g[f"mesh/{k}@{lev}"]
            assert a.shape == b.shape and np.array_equal(a, b), (case, lev, k)
        hang = m.get("hang", lev).reshape(3, -1)
        for i, k in enumerate(("hang_node", "hang_c0", "hang_c1")):
            assert np.array_equal(hang[i], g[f"mesh/{k}@{lev}"]), (case, lev, k)
        assert np.array_equal(m.get("T_bc", lev), g[f"mesh/T_bc@{lev}"].astype(np.int32))
        vbc = m.get("v_bc", lev).reshape(2, -1)
        assert np.array_equal(vbc[0], g[f"mesh/v_bc0@{lev}"].astype(np.int32))
        assert np.array_equal(vbc[1], g[f"mesh/v_bc1@{lev}"].astype(np.int32))


@pytest.mark.parametrize("case", CASES)
def test_geometry_bit_exact(case):
    g = golden(case)
    m = Mesh(Config.from_input(golden_input(case)))
    lev = m.max_level - 1
    X = m.get("X", lev).reshape(2, -1)
    assert np.array_equal(X[0], g[f"mesh/X0@{lev}"]) and np.array_equal(X[1], g[f"mesh/X1@{lev}"])
    assert np.array_equal(m.get("jacobi", lev), g[f"mesh/jacobi@{lev}"])
    assert np.array_equal(m.get("area", lev), g[f"mesh/area@{lev}"])
    vv = m.get("v_bc_val", lev).reshape(2, -1)
    assert np.array_equal(vv[0], g[f"mesh/v_bc_val0@{lev}"])
    assert np.array_equal(m.get("T_bc_val", lev), g[f"mesh/T_bc_val@{lev}"])


@pytest.mark.parametrize("case", ["cfg1_l5", "hang11_l6", "vc_l6"])
def test_seeded_initial_temperature(case):
    """T_ini=-2 seeded field equals the harness's T on every level (same Philox stream)."""
    g = golden(case)
    m = Mesh(Config.from_input(golden_input(case)))
    for k in g.files:
        if k.startswith("ops/T@"):
            lev = int(k.split("@")[1])
            if lev == m.max_level - 1:
                assert np.array_equal(m.initial_temperature(lev), g[k]), (case, lev)
