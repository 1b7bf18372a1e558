"""The node-block operator's structure built by the host mesh builder: each
node's matrix neighbours (the distinct nodes of the elements touching it,
ascending) and each element's corner-to-slot map.  The builder computes both
in node and element chunks on threads; on meshes large enough to be split
(hundreds of thousands of nodes: uniform, graded by |grad T|-style flags, and a
develop_mode pattern) they equal a numpy restatement from the connectivity."""
import numpy as np
import pytest
from conftest import golden_input

from mantle_convection_lab_gb300 import Config, Mesh
from mantle_convection_lab_gb300.api import NB_WIDTH


def cfg(level, dev=0):
    c = Config.from_input(golden_input("cfg1_l5"))
    c.level, c.mg_min_level, c.develop_mode = level, level - 2, dev
    return c


def uniform_leaves(F, base):
    return np.arange(0, 1 << (2 * F), 1 << (2 * (F - base)), dtype=np.int32)


def expected_neighbours(m):
    node = m.get("node")
    ienl = np.searchsorted(node, m.get("ien").reshape(4, -1))
    pairs = np.stack([np.concatenate([ienl[a] for a in range(4) for _ in range(4)]),
                      np.concatenate([ienl[b] for _ in range(4) for b in range(4)])], 1)
    uniq = np.unique(pairs, axis=0)                      # sorted by node, then neighbour
    counts = np.bincount(uniq[:, 0], minlength=node.size)
    slot = np.arange(uniq.shape[0]) - np.repeat(np.cumsum(counts) - counts, counts)
    out = np.full((node.size, NB_WIDTH), -1, np.int32)
    out[uniq[:, 0], slot] = uniq[:, 1]
    return out, ienl


def mesh(kind):
    if kind == "uniform":
        return Mesh(cfg(10))
    if kind == "graded":
        c = cfg(10)
        m = Mesh(c, leaves=uniform_leaves(9, 6))
        flags = (np.random.default_rng(5).random(m.nel) < 0.1).astype(np.uint8)
        return Mesh(c, leaves=m.amr_leaves(flags, 6, 9))
    return Mesh(cfg(10, 12))


@pytest.mark.parametrize("kind", ["uniform", "graded", "develop_mode_12"])
def test_neighbour_lists_and_slots(kind):
    m = mesh(kind)
    assert m.nno > 3 * 16384   # split over several threads
    want, ienl = expected_neighbours(m)
    nb = m.get("nb").reshape(m.nno, NB_WIDTH)
    np.testing.assert_array_equal(nb, want)
    ks = m.get("kslot").reshape(4, 4, m.nel)
    for a in range(4):
        for b in range(4):
            np.testing.assert_array_equal(nb[ienl[a], ks[a, b]], ienl[b])
