"""Checkpoint / restart (mclg_checkpoint_save, mclg_checkpoint_load,
mclg_restart): a run restarted from a checkpoint continues bit for bit as the
uninterrupted run -- the FP64 replica (its kept pressure), the converged
solver with its two-step extrapolation history, and a refined mesh rebuilt
from the checkpoint's leaves -- and damaged or foreign files are refused.
"""
import numpy as np
import pytest
from conftest import golden_input

from mantle_convection_lab_gb300 import Config, MclgError, Model, amr, learned
from mantle_convection_lab_gb300.api import BAD_INPUT, IO_ERROR

pytestmark = pytest.mark.gpu

FIELDS = ("T", "V0", "V1", "P", "d", "stress")


def _fields(m):
    return {k: m.get(k) for k in FIELDS}


def _run(cfg, n, leaves=None):
    m = Model(cfg, leaves=leaves)
    m.initial_temperature()
    for _ in range(n):
        m.step()
    return m


def _continues_exactly(cfg, tmp_path, before=2, after=2, leaves=None):
    with _run(cfg, before + after, leaves) as full:
        want, want_t = _fields(full), full.time()
    path = str(tmp_path / "state.ckp")
    with _run(cfg, before, leaves) as m:
        m.checkpoint(path)
    with Model(cfg, restart=path) as r:
        assert r.time()[0] == before
        for _ in range(after):
            r.step()
        got, got_t = _fields(r), r.time()
    assert got_t == want_t
    for k in FIELDS:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)


def test_replica_restart_is_bitwise(tmp_path):
    cfg = Config.from_input(golden_input("cfg1_l5"))
    cfg.zero_P = 0          # the pressure carries over between steps
    _continues_exactly(cfg, tmp_path)


def test_converged_restart_keeps_extrapolation_history(tmp_path):
    cfg = Config.from_input(learned.DEFAULT_INPUT)
    cfg.level = 7
    assert cfg.warm_start == 3 and cfg.precision == 1
    _continues_exactly(cfg, tmp_path, before=3, after=2)


def test_refined_mesh_restart(tmp_path):
    cfg = Config.from_input(amr.CFG2_INPUT)
    cfg.level = 8
    cfg.max_citcom_cycle, cfg.max_cg_cycle = 30, 100
    with Model(cfg, leaves=amr.uniform_leaves(cfg.level - 1, 5)) as m:
        m.initial_temperature()
        m.remesh(0.2, 5, 7)
        leaves = m.mesh("Mcode") >> 4
        nel = m.nel
    assert nel > 1 << 10
    _continues_exactly(cfg, tmp_path, before=1, after=1, leaves=leaves)


def test_load_refuses_foreign_and_damaged_files(tmp_path):
    cfg = Config.from_input(golden_input("cfg1_l5"))
    path = str(tmp_path / "a.ckp")
    with _run(cfg, 1) as m:
        m.checkpoint(path)
        other = Config.from_input(golden_input("hang11_l6"))
        with Model(other) as o:
            with pytest.raises(MclgError) as e:
                o.load_checkpoint(path)
            assert e.value.status == BAD_INPUT
        raw = bytearray(open(path, "rb").read())
        raw[len(raw) // 2] ^= 0x40
        bad = tmp_path / "b.ckp"
        bad.write_bytes(bytes(raw))
        with pytest.raises(MclgError) as e:
            m.load_checkpoint(str(bad))
        assert e.value.status == IO_ERROR
        short = tmp_path / "c.ckp"
        short.write_bytes(bytes(raw[:200]))
        with pytest.raises(MclgError) as e:
            m.load_checkpoint(str(short))
        assert e.value.status == IO_ERROR
