"""Grain-size rheology (grain_damage=1, Grain_size_evolution.c:3-152) in the
engine's step: the FP64 replica with the host grain-size routine after the
exponential viscosity, against the reference's own runs on single-level meshes
(tests/golden/gd_l5: cold top, the clip sets the viscosity near the top;
gdw_l5: warmer top, the grain size evolves and the clip acts at both ends).
Every step: velocity, pressure, d, stress, viscosity and temperature to 1e-8 and
the grain size to 1e-10 (its inputs are the engine's stress, which agrees with the
reference's to rounding, not bit for bit), Uzawa counts within one.  (The file sorts last: it is
the newest GPU test.)"""
import pytest
from conftest import golden, golden_input, rel

from mantle_convection_lab_gb300 import Config, MclgError, Model

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["gd_l5", "gdw_l5"])
def test_steps_match_reference(case):
    g = golden(case)
    with Model(Config.from_input(golden_input(case))) as m:
        m.initial_temperature()
        for s in g["series/steps"]:
            st = m.step()
            assert abs(st.uzawa_cycles - int(g["series/uzawa_cycles"][s])) <= 1, (s, st.uzawa_cycles)
            for f, key in (("V0", "V0"), ("V1", "V1"), ("P", "p"), ("d", "d"), ("stress", "stress"),
                           ("vis", "vis")):
                err = rel(m.get(f), g[f"step{s:04d}/{key}"])
                assert err < 1e-8, (s, f, err)
            assert rel(m.get("gs"), g[f"step{s:04d}/gs"]) < 1e-10, s
            assert rel(m.get("T"), g[f"heat{s:04d}/T"]) < 1e-8, s


def test_grain_runs_refuse_remesh_and_checkpoint(tmp_path):
    with Model(Config.from_input(golden_input("gd_l5"))) as m:
        m.initial_temperature()
        m.step()
        with pytest.raises(MclgError):
            m.remesh(0.2, 2, 4)
        with pytest.raises(MclgError):
            m.checkpoint(str(tmp_path / "g.ckp"))
