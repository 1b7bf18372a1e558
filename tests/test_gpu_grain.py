"""Grain-size rheology (grain_damage=1, Grain_size_evolution.c:3-152) in the
engine's step: the FP64 replica with the host grain-size routine after the
exponential viscosity, against the reference's own runs on single-level meshes
(tests/golden/gd_l5: cold top, the clip sets the viscosity near the top;
gdw_l5: warmer top, the grain size evolves and the clip acts at both ends).

Tolerances come from the oracle's own sensitivity
(tests/test_oracle_golden.py::test_grain_steps_are_ill_conditioned).  Step 0's
viscosity is the exponential law and the solve is well conditioned: every field
to 1e-8.  From step 1 on the viscosity spans the clip range [1e-3, 1e3] and the
Uzawa loop runs about 400 cycles of inner CG at its 2000-iteration cap; there
the reference's own arithmetic moves P by up to 3.9e-8 and V, d and stress by
up to 6.7e-9 when T is perturbed by 1e-15 relative, so a solver that sums in
another order is held to P 1e-7, V/d/stress 3e-8, grain size 5e-10 (envelope
6.8e-11), T and viscosity 1e-8.  Uzawa counts within one."""
import pytest
from conftest import golden, golden_input, rel

from mantle_convection_lab_gb300 import Config, MclgError, Model

pytestmark = pytest.mark.gpu

TOL_WELL = 1e-8                # step 0, and T / viscosity on every step
TOL_P, TOL_V, TOL_GS = 1e-7, 3e-8, 5e-10   # steps >= 1: the clip-range solves


@pytest.mark.parametrize("case", ["gd_l5", "gdw_l5"])
def test_steps_match_reference(case):
    g = golden(case)
    with Model(Config.from_input(golden_input(case))) as m:
        m.initial_temperature()
        for s in g["series/steps"]:
            st = m.step()
            assert abs(st.uzawa_cycles - int(g["series/uzawa_cycles"][s])) <= 1, (s, st.uzawa_cycles)
            tv, tp = (TOL_WELL, TOL_WELL) if s == 0 else (TOL_V, TOL_P)
            for f, key, tol in (("V0", "V0", tv), ("V1", "V1", tv), ("P", "p", tp), ("d", "d", tv),
                                ("stress", "stress", tv), ("vis", "vis", TOL_WELL)):
                err = rel(m.get(f), g[f"step{s:04d}/{key}"])
                assert err < tol, (s, f, err)
            assert rel(m.get("gs"), g[f"step{s:04d}/gs"]) < TOL_GS, s
            assert rel(m.get("T"), g[f"heat{s:04d}/T"]) < TOL_WELL, s


def test_grain_runs_refuse_remesh_and_checkpoint(tmp_path):
    with Model(Config.from_input(golden_input("gd_l5"))) as m:
        m.initial_temperature()
        m.step()
        with pytest.raises(MclgError):
            m.remesh(0.2, 2, 4)
        with pytest.raises(MclgError):
            m.checkpoint(str(tmp_path / "g.ckp"))
