"""The reference's own inner solvers solver="gs" and solver="mg", host side.

- the CPU oracle's gauss_seidel / multigrid (oracle/oracle.c, Solver.c:668-768,
  1866-1929) reproduces the reference's dumps bit for bit, Uzawa cycle counts
  included, on a uniform 16x16 mesh (mg and gs) and a 32x32 mesh with hanging
  nodes (mg);
- the engine's transfer maps (mclg_refmg.c, through the mesh API) equal the
  Python restatement of Connection.c:708-930 and 1051-1251 (oracle/mg_oracle.py)
  on uniform and refined meshes;
- the Gauss-Seidel wavefronts order every matrix neighbour pair the way the
  sequential sweep does;
- the coarse-level operators of the oracle match the reference's (every level
  is assembled each step from its own initial temperature).
"""
import numpy as np
import pytest
from conftest import golden, golden_input, rel

import mg_oracle
import oracle_port
from mantle_convection_lab_gb300 import Config, Mesh

TOL = 1e-12


@pytest.mark.parametrize("case", ["mg_l5", "gs_l5", "mg11_l6"])
def test_oracle_matches_reference(case):
    g = golden(case)
    o = oracle_port.Oracle(golden_input(case))
    for s in g["series/steps"]:
        st = o.step()
        assert st["uzawa_cycles"] == g["series/uzawa_cycles"][s]
        for f, key in (("V0", "V0"), ("V1", "V1"), ("P", "p"), ("d", "d")):
            assert rel(o.get(f), g[f"step{s:04d}/{key}"]) < TOL, (s, f)
        assert rel(o.get("T"), g[f"heat{s:04d}/T"]) < TOL
        assert rel(st["res_m"], g["series/res_m"][s]) < 1e-9
    o.close()


@pytest.mark.parametrize("case", ["mg_l5", "mg11_l6", "dev12_l7", "dev13_l8", "dev14_l7", "vc_l6"])
def test_maps_equal_restatement(case):
    c = Config.from_input(golden_input(case))
    m = Mesh(c)
    lo, fl = c.mg_min_level, m.max_level - 1
    arr = {lev: mg_oracle.level_arrays(m, lev) for lev in range(lo, fl + 1)}
    for lev in range(lo, fl + 1):
        if lev > lo:
            got = m.get("interp", lev)
            neq = got.size // 5
            n, src = mg_oracle.interp(arr[lev - 1], arr[lev], lev - 1)
            np.testing.assert_array_equal(got[:neq], n)
            np.testing.assert_array_equal(got[neq:].reshape(4, neq), src)
            # every free equation of the finer level receives an interpolated error
            assert (n > 0).all()
        if lev < fl:
            up_eq = m.get("project", lev)
            np.testing.assert_array_equal(up_eq, mg_oracle.project(arr[lev], arr[lev + 1]))
            assert (up_eq >= 0).all()
    for bad in (lo, fl + 1):
        with pytest.raises(Exception):
            m.get("interp", bad)
    with pytest.raises(Exception):
        m.get("project", fl)


@pytest.mark.parametrize("case", ["mg_l5", "mg11_l6", "dev13_l8"])
def test_gauss_seidel_wavefronts(case):
    """Row A reads the new value of each neighbour B < A and the old value of
    each neighbour C > A: wave(B) < wave(A) < wave(C) for every matrix entry."""
    c = Config.from_input(golden_input(case))
    m = Mesh(c)
    g = golden(case)
    for lev in range(c.mg_min_level, m.max_level):
        wave = m.get("gs_wave", lev)
        if f"ops/K_ptr@{lev}" not in g:
            continue
        ptr, col = g[f"ops/K_ptr@{lev}"], g[f"ops/K_col@{lev}"]
        idv = m.get("id", lev).reshape(2, -1)
        node_of = np.empty(int(ptr.size - 1), np.int64)
        for d in range(2):
            free = idv[d] >= 0
            node_of[idv[d][free]] = np.nonzero(free)[0]
        rows = np.repeat(np.arange(ptr.size - 1), np.diff(ptr))
        A, B = node_of[rows], node_of[col]
        below, above = B < A, B > A
        assert (wave[B[below]] < wave[A[below]]).all()
        assert (wave[B[above]] > wave[A[above]]).all()
        assert wave.max() < 3 * max(m.gnox, m.gnoz)


def test_oracle_coarse_operators():
    """Coarse K from each level's initial temperature (viscosity contrast 1e5)."""
    g = golden("vc_l6")
    c = Config.from_input(golden_input("vc_l6"))
    c.solver = b"mg"
    o = oracle_port.Oracle(c)
    o.assemble()
    m = o.mesh
    for k, lev in enumerate(range(c.mg_min_level, m.max_level - 1)):
        lv = o._lv[k]
        out = np.zeros(m.get("node", lev).size)
        oracle_port.lib().orc_get(lv, oracle_port.GET["vis"], oracle_port._p(out))
        assert rel(out, g[f"ops/vis@{lev}"]) < TOL
        x = np.ascontiguousarray(g[f"ops/probe_x@{lev}"])
        y = np.zeros(x.size)
        oracle_port.lib().orc_kmul(lv, oracle_port._p(x), oracle_port._p(y))
        assert rel(y, g[f"ops/Kx@{lev}"]) < TOL
    o.close()
