"""GPU path (libmclg.so through its C ABI) against the reference's own dumps.

Single operators (assembled K, F, G, G^T, BAB, heat K and C) must agree to
1e-12 relative L2; the Stokes solution, stress and temperature after each
time step to 1e-8 relative L2 (the parity bar for velocity, pressure and
temperature), with the Uzawa iteration count within one of the reference's.
"""
import os

import numpy as np
import pytest
from conftest import GOLDEN, golden, golden_input, rel

from mantle_convection_lab_gb300 import Config, Model

pytestmark = pytest.mark.gpu

OP_TOL = 1e-12
FIELD_TOL = 1e-8


def make(case):
    m = Model(Config.from_input(golden_input(case)))
    m.initial_temperature()
    return m


@pytest.mark.parametrize("case", ["cfg1_l5", "hang11_l6", "vc_l6", "dev13_l8", "dev14_l7"])
def test_stokes_operators(case):
    g = golden(case)
    with make(case) as m:
        lev = m.max_level - 1
        # the seeded field uses libm sin/cos: hosts may differ in the last bit
        assert rel(m.get("T"), g[f"ops/T@{lev}"]) < 1e-15
        m.buoyancy_force()
        m.viscosity()
        m.velocity_pressure_KGF_matrix()
        assert rel(m.get("vis"), g[f"ops/vis@{lev}"]) < OP_TOL
        assert rel(m.get("buoyancy"), g[f"ops/buoyancy@{lev}"]) < OP_TOL
        assert rel(m.get("F"), g[f"ops/F@{lev}"]) < OP_TOL
        assert rel(m.get("Kdiag"), g[f"ops/Kdiag@{lev}"]) < OP_TOL
        assert rel(m.get("BAB"), g[f"ops/BAB@{lev}"]) < OP_TOL
        assert rel(m.stokes_matvec(g[f"ops/probe_x@{lev}"]), g[f"ops/Kx@{lev}"]) < OP_TOL
        assert rel(m.stokes_G(g[f"ops/probe_p@{lev}"]), g[f"ops/Gp@{lev}"]) < OP_TOL
        assert rel(m.stokes_GT(g[f"ops/probe_x@{lev}"]), g[f"ops/GTx@{lev}"]) < OP_TOL


# Cases whose Uzawa loop stops at max_citcom_cycle before converging.  Their
# iterates depend on summation order: the CPU oracle with 16 threads moves
# dev14_l7 by 3e-5 from the reference.  They are held to 1e-5 instead, and
# dev14_l7, whose iterate moves by 1e-4 (V) and 8e-4 (P) when T moves by
# 1e-13 (test_oracle_golden.py::test_capped_dev14_iterate_is_ill_conditioned),
# to 2e-3.
CAPPED_TOL = 1e-5
ILL_TOL = 2e-3


@pytest.mark.parametrize("case,steps,tol", [("cfg1_l5", 4, FIELD_TOL), ("vc_l6", 3, FIELD_TOL),
                                            ("hang11v_l6", 2, CAPPED_TOL), ("dev12_l7", 1, CAPPED_TOL),
                                            ("dev13_l8", 1, CAPPED_TOL), ("dev14_l7", 1, ILL_TOL)])
def test_time_steps(case, steps, tol):
    g = golden(case)
    with make(case) as m:
        for s in range(steps):
            st = m.step()
            assert st.status in (0, 1), st.status
            assert abs(st.uzawa_cycles - int(g["series/uzawa_cycles"][s])) <= 1
            assert rel(st.dt, g["series/dt"][s]) < tol
            assert rel(st.model_time, g["series/model_time"][s]) < tol
            for f, k in (("V0", "V0"), ("V1", "V1"), ("P", "p"), ("d", "d"), ("stress", "stress")):
                e = rel(m.get(f), g[f"step{s:04d}/{k}"])
                assert e < tol, (case, s, f, e)
            e = rel(m.get("T"), g[f"heat{s:04d}/T"])
            assert e < tol, (case, s, "T", e)


def rel_nan(a, b):
    """Relative L2 over the finite entries; the NaN pattern itself must match.
    The reference's tau is NaN where cosh/sinh overflow (cell Peclet > 710)."""
    a, b = np.asarray(a), np.asarray(b)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    f = ~np.isnan(b)
    return rel(a[f], b[f])


@pytest.mark.parametrize("case", ["cfg1_l5", "hang11v_l6", "vc_l6"])
def test_heat_operators(case):
    """tau, heat F and the heat K, C products of the first step (Update_temperature.c)."""
    g = golden(case)
    with make(case) as m:
        m.step()
        h = "heat0000"
        assert rel_nan(m.get("tau0"), g[f"{h}/tau0"]) < FIELD_TOL
        assert rel_nan(m.get("tau1"), g[f"{h}/tau1"]) < FIELD_TOL
        assert rel_nan(m.get("heat_F"), g[f"{h}/heat_F"]) < FIELD_TOL
        x = g[f"{h}/heat_probe_x"]
        assert rel_nan(m.heat_matvec("K", x), g[f"{h}/HKx"]) < FIELD_TOL
        assert rel_nan(m.heat_matvec("C", x), g[f"{h}/HCx"]) < FIELD_TOL


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "cfg1_l7.npz")), reason="fixture not generated")
def test_configuration1_100_steps():
    """Configuration 1 as specified: 64x64, Ra=1e5, 100 steps, Jacobi-PCG, true residual 1e-8."""
    g = golden("cfg1_l7")
    keep = {int(k[4:8]) for k in g.files if k.startswith("step")}
    with make("cfg1_l7") as m:
        for s in range(100):
            st = m.step()
            assert st.res_momentum < 1e-8 and st.res_continuity < 1e-8
            if s in keep:
                for f, k in (("V0", "V0"), ("V1", "V1"), ("P", "p"), ("stress", "stress")):
                    assert rel(m.get(f), g[f"step{s:04d}/{k}"]) < FIELD_TOL, (s, f)
                assert rel(m.get("T"), g[f"heat{s:04d}/T"]) < FIELD_TOL, (s, "T")
        assert rel(st.model_time, g["series/model_time"][99]) < FIELD_TOL
