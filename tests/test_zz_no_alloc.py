"""The allocation-free Stokes solve against the regular one, through the C ABI.

mclg_solve_velocity_pressure_noalloc serves callers that must not allocate
device memory while they run (their host program hands out all device memory
up front, or their time loop cannot take cudaMalloc's latency and device
synchronisation).  It must give the same velocity, pressure and stress as
mclg_solve_velocity_pressure on the same state, on every call -- the array
it works in keeps the previous call's contents, so two calls in a row are
checked -- and must refuse meshes larger than its fixed scratch.

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
