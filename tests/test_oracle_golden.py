"""The CPU oracle (oracle/oracle.c) against the reference's own dumps.

With one thread the oracle sums in the reference's order; on these fixtures it
reproduces the reference bit for bit (the tolerance is only there for hosts
whose libm rounds exp/cosh/sinh differently).
"""
import numpy as np
import pytest
from conftest import golden, golden_input, rel

import oracle_port

TOL = 1e-12


@pytest.mark.parametrize("case,steps", [("cfg1_l5", 4), ("hang11v_l6", 1), ("vc_l6", 1), ("dev12_l7", 1)])
def test_oracle_steps(case, steps):
    g = golden(case)
    o = oracle_port.Oracle(golden_input(case))
    for s in range(steps):
        st = o.step()
        assert st["uzawa_cycles"] == g["series/uzawa_cycles"][s]
        # the reference also prints a count for initial_T_dot's solve before step 0
        assert st["heat_cg_cycles"] == g["series/heat_cg_cycles"][s + 1]
        assert rel(st["dt"], g["series/dt"][s]) < TOL
        assert rel(o.get("V0"), g[f"step{s:04d}/V0"]) < TOL
        assert rel(o.get("V1"), g[f"step{s:04d}/V1"]) < TOL
        assert rel(o.get("P"), g[f"step{s:04d}/p"]) < TOL
        assert rel(o.get("d"), g[f"step{s:04d}/d"]) < TOL
        assert rel(o.get("stress"), g[f"step{s:04d}/stress"]) < TOL
        assert rel(o.get("T"), g[f"heat{s:04d}/T"]) < TOL
        assert rel(st["res_m"], g["series/res_m"][s]) < 1e-6


@pytest.mark.parametrize("case", ["cfg1_l5", "hang11_l6", "vc_l6"])
def test_oracle_operators(case):
    g = golden(case)
    o = oracle_port.Oracle(golden_input(case))
    o.assemble()
    lev = o.mesh.max_level - 1
    assert rel(o.get("F"), g[f"ops/F@{lev}"]) < TOL
    assert rel(o.get("Kdiag"), g[f"ops/Kdiag@{lev}"]) < TOL
    assert rel(o.get("vis"), g[f"ops/vis@{lev}"]) < TOL
    assert rel(o.get("buoyancy"), g[f"ops/buoyancy@{lev}"]) < TOL
    assert rel(o.kmul(g[f"ops/probe_x@{lev}"]), g[f"ops/Kx@{lev}"]) < TOL
    assert rel(o.gmul(g[f"ops/probe_p@{lev}"]), g[f"ops/Gp@{lev}"]) < TOL
    assert rel(o.gtmul(g[f"ops/probe_x@{lev}"]), g[f"ops/GTx@{lev}"]) < TOL


def test_capped_dev14_iterate_is_ill_conditioned():
    """dev14_l7 stops at max_citcom_cycle=40 with every inner CG at its
    2000-iteration cap (accuracy=1e-20 is never met), so its iterate amplifies
    rounding: moving T by 1e-13 relative -- the size of the rounding in one
    sequential sum over its 3e4 unknowns -- moves V by ~1e-4 and P by ~1e-3.
    A solver that sums in another order can only be held to that envelope
    there, which is the tolerance the GPU parity test uses for this case."""
    g = golden("dev14_l7")
    o = oracle_port.Oracle(golden_input("dev14_l7"))
    T = o.mesh.initial_temperature()
    o.set_T(T * (1 + 1e-13 * np.random.default_rng(0).standard_normal(T.size)))
    st = o.step()
    assert st["uzawa_cycles"] == 40
    e = {k: rel(o.get(k), g[f"step0000/{kk}"]) for k, kk in (("V0", "V0"), ("V1", "V1"), ("P", "p"))}
    o.close()
    assert e["V0"] > 3e-5 and e["V1"] > 3e-5 and e["P"] > 3e-4, e
    assert max(e.values()) < 2e-3, e


def test_grain_steps_are_ill_conditioned():
    """From step 1 on, the grain-size runs solve with the viscosity spread over
    the clip range [1e-3, 1e3] and about 400 Uzawa cycles of inner CG at its
    2000-iteration cap.  Moving T by 1e-15 relative -- below the rounding of one
    summation -- leaves the viscosity unchanged to 1e-15 but moves the oracle's
    own P by more than 1e-8 (measured 1.3e-8 .. 3.9e-8 over seeds) and V by up
    to 7e-9.  That envelope, not the grain law, sets the GPU test's bars for
    these steps (P 1e-7, V/d/stress 3e-8)."""
    g = golden("gdw_l5")
    worst = {"P": 0.0, "V": 0.0, "vis": 0.0}
    for seed in (0, 3):
        o = oracle_port.Oracle(golden_input("gdw_l5"))
        T = o.mesh.initial_temperature()
        o.set_T(T * (1 + 1e-15 * np.random.default_rng(seed).standard_normal(T.size)))
        o.step()
        o.step()
        worst["P"] = max(worst["P"], rel(o.get("P"), g["step0001/p"]))
        worst["V"] = max(worst["V"], rel(o.get("V0"), g["step0001/V0"]), rel(o.get("V1"), g["step0001/V1"]))
        worst["vis"] = max(worst["vis"], rel(o.get("vis"), g["step0001/vis"]))
        o.close()
    assert worst["vis"] < 1e-15, worst
    assert 1e-8 < worst["P"] < 1e-7, worst
    assert worst["V"] < 3e-8, worst


@pytest.mark.parametrize("case,steps", [("gd_l5", 2), ("gdw_l5", 2)])
def test_oracle_grain_size(case, steps):
    """Grain-size rheology (grain_damage=1, Grain_size_evolution.c:3-152) on a
    single-level mesh: the grain size, the viscosity it sets (clipped to
    [lowest_vis, highest_vis]) and the fields of the steps built on it equal the
    reference's.  gd_l5 has a cold top (the grain size stays at 1e-3, the clip
    sets the viscosity within 200 km of the top); gdw_l5 a warmer top, where
    the grain size evolves."""
    g = golden(case)
    o = oracle_port.Oracle(golden_input(case))
    for s in range(steps):
        st = o.step()
        assert st["uzawa_cycles"] == g["series/uzawa_cycles"][s]
        for name, key in (("gs", "gs"), ("vis", "vis"), ("V0", "V0"), ("V1", "V1"), ("P", "p"), ("d", "d"),
                          ("stress", "stress")):
            assert rel(o.get(name), g[f"step{s:04d}/{key}"]) < TOL, (s, name)
        assert rel(o.get("T"), g[f"heat{s:04d}/T"]) < TOL
    if case == "gdw_l5":   # the grain size did evolve, and the clip is active at both ends
        assert g[f"step{steps - 1:04d}/gs"].min() < 1e-3
        v = g[f"step{steps - 1:04d}/vis"]
        assert v.min() == 1e-3 and v.max() == 1e3
