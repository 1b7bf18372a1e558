"""Mesh numbering and hanging-node detection on the device (k_mesh.cu)
against the host builder (Construct_ien_id_lm.c:3-196, Connection.c:59-276,
Boundary_condition.c:10-110): every array of every level -- Mcode, node list
and id table, ien, local ien, levels, velocity and heat equation numbers, BC
codes and values, coordinates, geometry, node->element map, hanging nodes and
their parents, neighbour lists, element slot map, fine cell map -- equal byte
for byte, on uniform, graded and random trees, at configuration 2's size, with
other boundary codes and above the host's 4M-id table limit.
"""
import numpy as np
import pytest
from conftest import golden_input

from mantle_convection_lab_gb300 import Config, MclgError, Mesh, amr

pytestmark = pytest.mark.gpu


def cfg(level, min_level=2):
    c = Config.from_input(golden_input("cfg1_l5"))
    c.level, c.mg_min_level, c.develop_mode = level, min_level, 0
    return c


def uniform(F, base):
    return np.arange(0, 1 << (2 * F), 1 << (2 * (F - base)), dtype=np.int32)


def refined(c, F, base, target, density, seed, start=None):
    m = Mesh(c, leaves=uniform(F, base) if start is None else start)
    flags = (np.random.default_rng(seed).random(m.nel) < density).astype(np.uint8)
    return m.amr_leaves(flags, base, target)


def check(c, leaves):
    host = Mesh(c, leaves=leaves)
    dev = Mesh(c, leaves=leaves, device=True)
    assert dev.diff(host) is None, dev.diff(host)
    return host


@pytest.mark.parametrize("F,base,target,density,seed", [
    (6, 3, 6, 0.0, 0), (6, 3, 6, 0.1, 1), (6, 2, 6, 0.2, 2), (6, 1, 6, 0.5, 3), (6, 3, 6, 1.0, 4),
    (7, 4, 7, 0.2, 5), (8, 3, 8, 0.05, 6),
])
def test_device_numbering_equals_host(F, base, target, density, seed):
    c = cfg(F + 1)
    host = check(c, refined(c, F, base, target, density, seed))
    if density > 0 and density < 1:
        assert host.nh > 0


def test_graded_trees_refined_again():
    """A graded tree refined once more (the second remesh of a run)."""
    c = cfg(8, 3)
    first = refined(c, 7, 3, 6, 0.15, 11)
    check(c, first)
    check(c, refined(c, 7, 3, 7, 0.1, 12, start=first))


def test_other_boundary_codes():
    """Fixed velocities on the side walls and fixed temperature on them, so
    that every branch of the BC codes and of both equation numberings runs."""
    c = cfg(7)
    c.lef_v_bc, c.rig_v_bc = b"VV", b"VS"
    c.lef_T_bc, c.rig_T_bc, c.bot_T_bc = b"T", b"T", b"F"
    c.lef_T_bc_val, c.rig_T_bc_val = 0.25, 0.75
    host = check(c, refined(c, 6, 3, 6, 0.1, 21))
    assert host.neq < 2 * host.nno and host.heat_neq < host.nno


def test_configuration_2_size():
    c = Config.from_input(amr.CFG2_INPUT)
    c.precision = 1
    check(c, refined(c, c.level - 1, 7, 10, 0.05, 31))


def test_beyond_the_host_id_table():
    """4097^2 node ids: the host sorts and binary-searches instead of keeping a
    direct table; the device result must still be the same."""
    c = cfg(13, 8)
    check(c, refined(c, 12, 6, 9, 0.05, 41))


def test_rejects_a_list_that_is_not_a_quadtree():
    c = cfg(6)
    bad = uniform(5, 3).copy()
    bad[1] += 1                       # a gap of 17 fine cells
    with pytest.raises(MclgError):
        Mesh(c, leaves=bad, device=True)
