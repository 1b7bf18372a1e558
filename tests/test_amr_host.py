"""|grad T| refinement on the host, against the numpy oracle (oracle/amr_oracle.py).

- a mesh built from a leaf list equals the develop_mode mesh with the same
  leaves, array for array (so leaf-built meshes inherit the bit-exact pinning
  of the develop_mode meshes against the reference);
- the refined tree from given flags equals the oracle's, leaf for leaf, and is
  2:1 balanced with the flagged regions at the target level;
- the bilinear transfer equals the oracle's and is exact for bilinear fields.
"""
import numpy as np
import pytest
from conftest import golden_input

import amr_oracle as ao
from mantle_convection_lab_gb300 import Config, MclgError, Mesh


def cfg(level=7, dev=0):
    c = Config.from_input(golden_input("cfg1_l5"))
    c.level, c.mg_min_level, c.develop_mode = level, 2, dev
    return c


def uniform_leaves(F, base):
    return np.arange(0, 1 << (2 * F), 1 << (2 * (F - base)), dtype=np.int32)


@pytest.mark.parametrize("dev,level", [(11, 6), (12, 7), (13, 8), (14, 7)])
def test_leaf_built_mesh_equals_pattern_mesh(dev, level):
    c = cfg(level, dev)
    a = Mesh(c)
    b = Mesh(c, leaves=a.get("Mcode") >> 4)
    for k in ("Mcode", "node", "ien", "id", "heat_id", "lm", "hang", "v_bc", "T_bc"):
        np.testing.assert_array_equal(a.get(k), b.get(k), err_msg=k)
    for lev in range(2, level):
        np.testing.assert_array_equal(a.get("Mcode", lev), b.get("Mcode", lev))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_refined_tree_equals_oracle(seed):
    F, base, target = 6, 3, 6
    c = cfg(F + 1)
    m = Mesh(c, leaves=uniform_leaves(F, base))
    assert m.nel == 64
    rng = np.random.default_rng(seed)
    flg = (rng.random(m.nel) < 0.15).astype(np.uint8)
    leaves = m.amr_leaves(flg, base, target)
    want, lv = ao.build_leaves(m.get("Mcode"), flg, F, base, target)
    np.testing.assert_array_equal(leaves, want)
    # 2:1 balance over edges and corners
    p = np.pad(lv, 1, constant_values=-10)
    for dx in (-1, 0, 1):
        for dz in (-1, 0, 1):
            q = p[1 + dx:1 + dx + lv.shape[0], 1 + dz:1 + dz + lv.shape[1]]
            assert (np.abs(q - lv)[q >= 0] <= 1).all()
    # flagged regions refined fully
    for e in np.nonzero(flg)[0]:
        x0, z0 = ao.demorton(int(m.get("Mcode")[e]) >> 4)
        s = 1 << (F - base)
        assert (lv[x0:x0 + s, z0:z0 + s] == target).all()
    # the new tree builds a mesh, with hanging nodes where levels meet
    r = Mesh(c, leaves=leaves)
    assert r.nel == leaves.size and r.nh > 0


def test_second_refinement_coarsens_back():
    F, base, target = 6, 3, 5
    c = cfg(F + 1)
    m = Mesh(c, leaves=uniform_leaves(F, base))
    flg = np.zeros(m.nel, np.uint8)
    flg[:4] = 1
    r = Mesh(c, leaves=m.amr_leaves(flg, base, target))
    # nothing flagged on the refined mesh: back to the base grid
    back = r.amr_leaves(np.zeros(r.nel, np.uint8), base, target)
    np.testing.assert_array_equal(back, uniform_leaves(F, base))


def test_transfer_equals_oracle_and_is_exact_for_bilinear_fields():
    F, base = 6, 3
    c = cfg(F + 1)
    m = Mesh(c, leaves=uniform_leaves(F, base))
    flg = np.zeros(m.nel, np.uint8)
    flg[[5, 6, 20, 40]] = 1
    r = Mesh(c, leaves=m.amr_leaves(flg, base, 6))
    X = m.get("X").reshape(2, -1)
    T = 0.3 + 0.7 * X[0] - 1.1 * X[1] + 0.5 * X[0] * X[1]
    got = m.transfer(T, r)
    np.testing.assert_array_equal(got, ao.transfer(m, T, r))
    Y = r.get("X").reshape(2, -1)
    want = 0.3 + 0.7 * Y[0] - 1.1 * Y[1] + 0.5 * Y[0] * Y[1]
    assert np.abs(got - want).max() < 1e-14
    assert np.abs(r.transfer(want, m) - T).max() < 1e-14


def test_bad_leaf_lists_are_rejected():
    c = cfg(6)
    with pytest.raises(MclgError):
        Mesh(c, leaves=np.array([0, 16, 8], np.int32))        # not increasing
    with pytest.raises(MclgError):
        Mesh(c, leaves=np.array([0], np.int32))               # too few
