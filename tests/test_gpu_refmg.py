"""The reference's own inner solvers on the GPU: solver="gs" (gauss_seidel,
Solver.c:1866-1929) and solver="mg" (multigrid, Solver.c:668-768), inside the
FP64 Uzawa replica, against the reference's dumps and the CPU oracle.

- fields after every step agree with the reference's to 1e-8 relative L2 and
  the Uzawa cycle counts to within one (the GPU assembles K with fused
  multiply-adds, the reference without, so the operators differ in the last
  bits; the solvers themselves sum in the reference's order);
- each level of the hierarchy holds the reference's viscosity and K, from the
  level's own initial temperature;
- meshes beyond the fixtures (viscosity contrast 1e5, 2:1 refinement) agree
  with the CPU oracle, which reproduces the reference bit for bit;
- the allocation-free entry point runs the same solver.
"""
import numpy as np
import pytest
from conftest import golden, golden_input, rel

import oracle_port
from mantle_convection_lab_gb300 import Config, MclgError, Model
from mantle_convection_lab_gb300.api import BAD_INPUT

pytestmark = pytest.mark.gpu

OP_TOL = 1e-12
FIELD_TOL = 1e-8


@pytest.mark.parametrize("case", ["mg_l5", "gs_l5", "mg11_l6"])
def test_steps_match_reference(case):
    g = golden(case)
    with Model(Config.from_input(golden_input(case))) as m:
        m.initial_temperature()
        for s in g["series/steps"]:
            st = m.step()
            assert abs(st.uzawa_cycles - int(g["series/uzawa_cycles"][s])) <= 1, (s, st.uzawa_cycles)
            assert st.cg_cycles > 0
            for f, key in (("V0", "V0"), ("V1", "V1"), ("P", "p"), ("d", "d"), ("stress", "stress")):
                err = rel(m.get(f), g[f"step{s:04d}/{key}"])
                assert err < FIELD_TOL, (s, f, err)
            assert rel(m.get("T"), g[f"heat{s:04d}/T"]) < FIELD_TOL
            assert abs(st.res_momentum - g["series/res_m"][s]) < 1e-6 * g["series/res_m"][s] + 1e-12


@pytest.mark.parametrize("case,solver", [("mg11_l6", "mg"), ("vc_l6", "mg")])
def test_coarse_levels_hold_reference_operators(case, solver):
    g = golden(case)
    c = Config.from_input(golden_input(case))
    c.solver = solver.encode()
    with Model(c) as m:
        m.initial_temperature()
        for lev in range(c.mg_min_level, m.max_level - 1):
            assert rel(m.get("T", lev), g[f"ops/T@{lev}"]) < 1e-15
            assert rel(m.get("vis", lev), g[f"ops/vis@{lev}"]) < OP_TOL
            assert rel(m.stokes_matvec(g[f"ops/probe_x@{lev}"], lev), g[f"ops/Kx@{lev}"]) < OP_TOL


def _oracle_case(case, solver, **over):
    c = Config.from_input(golden_input(case))
    c.solver = solver.encode()
    for k, v in over.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("case,solver,steps,over", [
    ("vc_l6", "mg", 1, {"max_citcom_cycle": 150}),                       # viscosity contrast 1e5
    ("vc_l6", "gs", 1, {"max_citcom_cycle": 60}),
    ("dev12_l7", "mg", 1, {"mg_min_level": 4, "max_citcom_cycle": 80}),   # 2:1 refinement band
    ("mg_l5", "mg", 2, {"mg_cycle": 3, "mg_finest_iteration": 2, "mg_coarse_iteration": 6}),
])
def test_matches_oracle(case, solver, steps, over):
    c = _oracle_case(case, solver, **over)
    o = oracle_port.Oracle(c)
    with Model(c) as m:
        m.initial_temperature()
        for s in range(steps):
            st = m.step()
            ost = o.step()
            assert abs(st.uzawa_cycles - ost["uzawa_cycles"]) <= 1, (s, st.uzawa_cycles, ost["uzawa_cycles"])
            for f in ("V0", "V1", "P", "T"):
                err = rel(m.get(f), o.get(f))
                assert err < FIELD_TOL, (s, f, err)
    o.close()


def test_noalloc_runs_the_same_solver():
    with Model(Config.from_input(golden_input("mg11_l6"))) as m:
        m.initial_temperature()
        m.buoyancy_force()
        m.viscosity()
        m.velocity_pressure_KGF_matrix()
        ref_st = m.solve_velocity_pressure()
        ref = {k: m.get(k) for k in ("V0", "V1", "P")}
        st = m.solve_velocity_pressure_noalloc()
        assert (st.uzawa_cycles, st.cg_cycles) == (ref_st.uzawa_cycles, ref_st.cg_cycles)
        for k in ref:
            assert rel(m.get(k), ref[k]) < 1e-14


def test_mg_needs_two_levels():
    c = Config.from_input(golden_input("mg_l5"))
    c.mg_min_level = c.level - 1
    with pytest.raises(MclgError) as e:
        Model(c)
    assert e.value.status == BAD_INPUT and "mg_min_level" in str(e.value)
