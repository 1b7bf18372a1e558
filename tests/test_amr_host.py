"""|grad T| refinement on the host, against the numpy oracle (oracle/amr_oracle.py).

- a mesh built from a leaf list equals the develop_mode mesh with the same
  leaves, array for array (so leaf-built meshes inherit the bit-exact pinning
  of the develop_mode meshes against the reference);
- the refined tree from given flags equals the oracle's, leaf for leaf, and is
  2:1 balanced with the flagged regions at the target level;
- the bilinear transfer equals the oracle's and is exact for bilinear fields;
- the element-field (pressure) transfer is the area mean of the old field over
  each new element: equal to a fine-cell raster mean in numpy, exact where the
  new mesh refines, conserving the field's integral, averaging a checkerboard
  over refined children to zero.
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


def _compact16(v):
    v = v & 0x55555555
    v = (v | (v >> 1)) & 0x33333333
    v = (v | (v >> 2)) & 0x0F0F0F0F
    v = (v | (v >> 4)) & 0x00FF00FF
    v = (v | (v >> 8)) & 0x0000FFFF
    return v


def _squares(m):
    """Per finest-level element: fine-cell origin (x0, z0) and side s."""
    M = m.get("Mcode").astype(np.int64)
    F = m.max_level - 1
    code = M >> 4
    return _compact16(code >> 1), _compact16(code), 1 << (F - (M & 15))


def _raster_mean(src, P, dst):
    """The area mean of src's element field P over each element of dst, by
    painting P on the finest cells and averaging."""
    F = src.max_level - 1
    grid = np.zeros((1 << F, 1 << F))
    for e, (x, z, s) in enumerate(zip(*_squares(src))):
        grid[x:x + s, z:z + s] = P[e]
    return np.array([grid[x:x + s, z:z + s].mean() for x, z, s in zip(*_squares(dst))])


def _graded(c, F, base, seed, density):
    m = Mesh(c, leaves=uniform_leaves(F, base))
    flg = (np.random.default_rng(seed).random(m.nel) < density).astype(np.uint8)
    return Mesh(c, leaves=m.amr_leaves(flg, base, F))


@pytest.mark.parametrize("seed", [0, 1])
def test_element_transfer_is_the_area_mean(seed):
    F, base = 6, 2
    c = cfg(F + 1)
    a, b = _graded(c, F, base, 10 + seed, 0.1), _graded(c, F, base, 20 + seed, 0.1)
    P = np.random.default_rng(seed).standard_normal(a.nel)
    got = a.transfer_elem(P, b)
    want = _raster_mean(a, P, b)
    assert np.abs(got - want).max() <= 1e-14 * np.abs(P).max()
    # the integral of the field is kept
    ia, ib = (a.get("area") * P).sum(), (b.get("area") * got).sum()
    assert abs(ia - ib) <= 1e-13 * (a.get("area") * np.abs(P)).sum()
    # onto the same mesh it is the identity
    np.testing.assert_array_equal(a.transfer_elem(P, a), P)


def test_element_transfer_is_exact_where_the_new_mesh_refines():
    F, base = 6, 3
    c = cfg(F + 1)
    coarse = Mesh(c, leaves=uniform_leaves(F, base))
    fine = _graded(c, F, base, 3, 0.3)
    P = np.random.default_rng(3).standard_normal(coarse.nel)
    got = coarse.transfer_elem(P, fine)
    # every new element lies in one old element and takes its value, bit for bit
    xs, zs, ss = _squares(coarse)
    owner = np.empty((1 << F, 1 << F), np.int64)
    for e, (x, z, s) in enumerate(zip(xs, zs, ss)):
        owner[x:x + s, z:z + s] = e
    x2, z2, _ = _squares(fine)
    np.testing.assert_array_equal(got, P[owner[x2, z2]])


def test_element_transfer_averages_a_checkerboard_away():
    F, base = 6, 3
    c = cfg(F + 1)
    fine = _graded(c, F, base, 4, 0.3)
    coarse = Mesh(c, leaves=uniform_leaves(F, base))
    x, z, s = _squares(fine)
    P = np.where(((x // s) + (z // s)) % 2 == 0, 1.0, -1.0)   # alternating over siblings of one size
    got = fine.transfer_elem(P, coarse)
    # the base elements split into children of a single size average to exactly 0
    split = []
    for x0, z0, w in zip(*_squares(coarse)):
        inside = s[(x >= x0) & (x < x0 + w) & (z >= z0) & (z < z0 + w)]
        split.append(inside.size > 1 and np.unique(inside).size == 1)
    split = np.array(split)
    assert split.any()
    np.testing.assert_array_equal(got[split], 0.0)


def test_element_transfer_rejects_mismatched_meshes():
    c6, c7 = cfg(6), cfg(7)
    a, b = Mesh(c6, leaves=uniform_leaves(5, 3)), Mesh(c7, leaves=uniform_leaves(6, 3))
    with pytest.raises(MclgError):
        a.transfer_elem(np.zeros(a.nel), b)                   # different finest level
    with pytest.raises(MclgError):
        a.transfer_elem(np.zeros(a.nel + 1), a)               # wrong field size


def test_transfers_on_meshes_split_across_threads():
    """Both transfers on meshes of over 100 000 nodes and elements (built in
    chunks on threads): bilinear fields move exactly, element fields by their area
    mean."""
    F, base = 9, 6
    c = cfg(F + 1)
    a, b = _graded(c, F, base, 31, 0.3), _graded(c, F, base, 32, 0.3)
    assert min(a.nno, b.nno, a.nel, b.nel) > 2 * 16384
    X = a.get("X").reshape(2, -1)
    T = 0.3 + 0.7 * X[0] - 1.1 * X[1] + 0.5 * X[0] * X[1]
    Y = b.get("X").reshape(2, -1)
    want = 0.3 + 0.7 * Y[0] - 1.1 * Y[1] + 0.5 * Y[0] * Y[1]
    assert np.abs(a.transfer(T, b) - want).max() < 1e-13
    P = np.random.default_rng(7).standard_normal(a.nel)
    got = a.transfer_elem(P, b)
    assert np.abs(got - _raster_mean(a, P, b)).max() <= 1e-14 * np.abs(P).max()


def test_mesh_diff_names_the_first_differing_array():
    """mclg_mesh_diff, which the device-numbering tests use: equal builds give
    None; a different boundary code shows up in the arrays it changes."""
    c = cfg(7)
    lv = uniform_leaves(6, 3)
    a, b = Mesh(c, leaves=lv), Mesh(c, leaves=lv)
    assert a.diff(b) is None
    c2 = cfg(7)
    c2.lef_T_bc_val = c.lef_T_bc_val + 0.5
    assert Mesh(c2, leaves=lv).diff(a) == "level 2 T_bc_val"
    c2.lef_T_bc = b"T"
    assert Mesh(c2, leaves=lv).diff(a) == "level 2 sizes"      # fewer heat equations


def test_device_numbering_fails_loudly_without_a_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present: tests/test_gpu_mesh_numbering.py covers it")
    with pytest.raises(MclgError):
        Mesh(cfg(7), leaves=uniform_leaves(6, 3), device=True)


@pytest.mark.parametrize("bad", ["decreasing", "out_of_range", "one_leaf"])
def test_leaf_list_checks(bad):
    """The leaf-list checks shared by the host and the device builders."""
    c = cfg(7)
    lv = uniform_leaves(6, 3)
    if bad == "decreasing":
        lv = lv[::-1].copy()
    elif bad == "out_of_range":
        lv = lv.copy()
        lv[-1] = 1 << 12
    else:
        lv = lv[:1].copy()
    with pytest.raises(MclgError):
        Mesh(c, leaves=lv)
