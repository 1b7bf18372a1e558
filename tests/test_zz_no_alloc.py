"""The allocation-free Stokes solve against the regular one, through the C ABI.

mclg_solve_velocity_pressure_noalloc serves callers that must not allocate
device memory while they run (their host program hands out all device memory
up front, or their time loop cannot take cudaMalloc's latency and device
synchronisation).  It must give the same velocity, pressure and stress as
mclg_solve_velocity_pressure on the same state, on every call -- the array
it works in keeps the previous call's contents, so two calls in a row are
checked -- and must refuse meshes larger than its fixed scratch.

The first test uses the fixtures' zero_P=1, so each solve starts from p = 0
and both entry points see the same start on every call.  With zero_P=0 the
pressure is kept from one solve to the next; that case is checked by two
models run in lockstep, one solving with each entry point.

This file is named to be collected last.
"""
import numpy as np
import pytest
from conftest import golden_input, rel

from mantle_convection_lab_gb300 import Config, MclgError, Model
from mantle_convection_lab_gb300.api import BAD_INPUT

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-8


def _state(m):
    return {k: m.get(k) for k in ("V0", "V1", "P", "d", "stress")}


@pytest.mark.parametrize("case", ["cfg1_l5", "hang11v_l6"])
def test_noalloc_matches_regular_solve(case):
    with Model(Config.from_input(golden_input(case))) as m:
        m.initial_temperature()
        m.buoyancy_force()
        m.viscosity()
        m.velocity_pressure_KGF_matrix()
        ref_st = m.solve_velocity_pressure()
        ref = _state(m)
        for call in range(2):
            st = m.solve_velocity_pressure_noalloc()
            got = _state(m)
            assert st.uzawa_cycles == ref_st.uzawa_cycles, call
            assert st.cg_cycles == ref_st.cg_cycles, call
            for k in ref:
                assert rel(got[k], ref[k]) < FIELD_TOL, (call, k)


def test_noalloc_keeps_pressure_like_regular_solve():
    """zero_P=0: each solve starts from the previous pressure.  Two models from
    the same input, one calling the regular solve and one the allocation-free
    solve, stay equal over two full steps (solve and temperature update)."""
    cfg = Config.from_input(golden_input("cfg1_l5"))
    cfg.zero_P = 0
    with Model(cfg) as a, Model(cfg) as b:
        a.initial_temperature()
        b.initial_temperature()
        for call in range(2):
            sts = []
            for m, solve in ((a, a.solve_velocity_pressure), (b, b.solve_velocity_pressure_noalloc)):
                m.buoyancy_force()
                m.viscosity()
                m.velocity_pressure_KGF_matrix()
                sts.append(solve())
                m.update_temperature()
            assert sts[0].uzawa_cycles == sts[1].uzawa_cycles, call
            assert sts[0].cg_cycles == sts[1].cg_cycles, call
            ra, rb = _state(a), _state(b)
            for k in ra:
                assert rel(rb[k], ra[k]) < FIELD_TOL, (call, k)
            assert rel(b.get("T"), a.get("T")) < FIELD_TOL, call


def test_noalloc_rejects_large_mesh():
    cfg = Config.from_input(golden_input("cfg1_l5"))
    cfg.level = 9   # 256 x 256: 66049 nodes, beyond the fixed scratch
    cfg.mg_min_level = 7
    with Model(cfg) as m:
        m.initial_temperature()
        m.buoyancy_force()
        m.viscosity()
        m.velocity_pressure_KGF_matrix()
        with pytest.raises(MclgError) as e:
            m.solve_velocity_pressure_noalloc()
        assert e.value.status == BAD_INPUT
        assert "allocation-free limit" in str(e.value)
