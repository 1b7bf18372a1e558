"""Batched ensembles (mclg_ensemble_*): one solver launch for many models.

- every member of a batch reaches the same solution as the same model
  stepped alone (the batched solve differs only in summation order);
- a member configured like the reference's 16x16 case matches the
  reference's own fields, so the batched path is pinned to the oracle too;
- the API rejects members it cannot batch.
"""
import numpy as np
import pytest
from conftest import golden, golden_input, rel

from mantle_convection_lab_gb300 import Config, Ensemble, MclgError, Model, ensemble
from mantle_convection_lab_gb300.api import BAD_INPUT

pytestmark = pytest.mark.gpu


def test_batch_matches_members_stepped_alone():
    cfgs = ensemble.configs(6, seed=1, sizes=(32, 64))
    with Ensemble(cfgs) as e:
        e.initial_temperature()
        for _ in range(4):
            stats = e.step()
            for s in stats:
                assert s.status == 0 and max(s.res_momentum, s.res_continuity) < 1e-8
        got = [(m.get("V0"), m.get("V1"), m.get("T"), m.stokes_G(m.get("P"))) for m in e.members]
    for i, c in enumerate(cfgs):
        with Model(c) as m:
            m.initial_temperature()
            for _ in range(4):
                m.step()
            want = (m.get("V0"), m.get("V1"), m.get("T"), m.stokes_G(m.get("P")))
        for k, tol in zip(("V0", "V1", "T", "Gp"), (1e-8, 1e-8, 1e-10, 1e-7)):
            e_ = rel(got[i][("V0", "V1", "T", "Gp").index(k)], want[("V0", "V1", "T", "Gp").index(k)])
            assert e_ < tol, (i, k, e_)


def _cfg1_converged():
    c = Config.from_input(golden_input("cfg1_l5"))
    c.precision, c.stokes_method, c.warm_start = 1, 1, 3
    c.stokes_rtol, c.outer_rtol, c.max_outer, c.max_refine, c.mg_coarse = 1e-8, 3e-3, 1000, 20, 2
    return c


def test_batch_member_matches_reference():
    g = golden("cfg1_l5")
    other = ensemble.configs(3, seed=2, sizes=(32,))
    with Ensemble([_cfg1_converged()] + other) as e:
        e.initial_temperature()
        m = e.members[0]
        for s in range(4):
            e.step()
            for f in ("V0", "V1"):
                err = rel(m.get(f), g[f"step{s:04d}/{f}"])
                assert err < 1e-8, (s, f, err)
            assert rel(m.get("T"), g[f"heat{s:04d}/T"]) < 1e-8


def test_batch_rejects_members_it_cannot_batch():
    replica = Config.from_input(golden_input("cfg1_l5"))        # precision=fp64: the replica, not batchable
    with pytest.raises(MclgError) as ex:
        Ensemble([_cfg1_converged(), replica])
    assert ex.value.status == BAD_INPUT
    tall = _cfg1_converged()
    tall.model_height = 2.0                                     # another element aspect ratio
    with pytest.raises(MclgError) as ex:
        Ensemble([_cfg1_converged(), tall])
    assert ex.value.status == BAD_INPUT


def test_refined_members_match_models_stepped_alone():
    """Refined members (of up to 2^20 nodes) are solved by one batched launch of
    the refined-mesh solver, a model per cluster; the summation order differs
    from a model stepped alone: V to 1e-8, T to 1e-10."""
    cfgs = ensemble.amr_configs(4, seed=3, sizes=(32, 64)) + ensemble.amr_configs(1, seed=7, sizes=(128,))
    levels = [0, 1, 2, 1, 2]
    with Ensemble(cfgs, levels) as e:
        e.initial_temperature()
        refined = [m.nh > 0 or m.nel != (1 << (2 * (c.level - 1))) for m, c in zip(e.members, cfgs)]
        assert refined == [False, True, True, True, True]
        leaves = [m.mesh("Mcode") >> 4 for m in e.members]
        for _ in range(3):
            st = e.step()
            for s in st:
                assert s.status == 0 and max(s.res_momentum, s.res_continuity) < 1e-8
            assert st[0].solver_kernel_launches == 2   # the uniform batch and the refined batch
        got = [(m.get("V0"), m.get("T")) for m in e.members]
    for i in (1, 2, 3, 4):
        c = cfgs[i]
        c.level += levels[i]
        with Model(c, leaves=leaves[i]) as m:
            m.initial_temperature()
            for _ in range(3):
                m.step()
            assert rel(got[i][0], m.get("V0")) < 1e-8 and rel(got[i][1], m.get("T")) < 1e-10, i


def test_graph_replay_matches_members_stepped_alone():
    """From step 7 on (after the cluster-size autotuner) the step is replayed as one
    CUDA graph; the members still match themselves stepped alone."""
    cfgs = ensemble.configs(3, seed=5, sizes=(32,))
    steps = 11
    with Ensemble(cfgs) as e:
        e.initial_temperature()
        used = []
        for _ in range(steps):
            for s in e.step():
                assert s.status == 0 and max(s.res_momentum, s.res_continuity) < 1e-8
            used.append(e.graph)
        assert used[:7] == [False] * 7 and all(used[8:]), used
        got = [(m.get("V0"), m.get("T")) for m in e.members]
    for i, c in enumerate(cfgs):
        with Model(c) as m:
            m.initial_temperature()
            for _ in range(steps):
                m.step()
            assert rel(got[i][0], m.get("V0")) < 1e-8 and rel(got[i][1], m.get("T")) < 1e-10
