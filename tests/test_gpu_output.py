"""Asynchronous output (mclg_output_async / mclg_output_wait, and mclg_step's
output): the files match Output.c's text byte for byte for the model's own
fields, several outputs can be in flight while the model steps on, the binary
side-car holds every field at full precision, and write errors come back.
"""
import os

import numpy as np
import pytest
from conftest import golden, golden_input

from mantle_convection_lab_gb300 import Config, MclgError, Mesh, Model
from mantle_convection_lab_gb300.api import IO_ERROR

pytestmark = pytest.mark.gpu

NAMES = ("coord", "temperature", "stress", "viscosity", "velocity")


def _fields(m):
    return {k: m.get(k) for k in ("T", "V0", "V1", "stress", "vis", "P")}


def _same_as_sync_writer(mesh, tmp_path, step, f, got_dir):
    ref_dir = tmp_path / f"sync{step}"
    mesh.write_output(str(ref_dir), step, f["T"], f["V0"], f["V1"], f["stress"], f["vis"])
    for n in NAMES:
        rel_path = f"{step:07d}/{n}.0.{step:07d}"
        assert (got_dir / rel_path).read_bytes() == (ref_dir / rel_path).read_bytes(), (step, n)


def test_step_output_is_the_text_of_the_models_fields(tmp_path):
    cfg = Config.from_input(golden_input("cfg1_l5"))
    out = tmp_path / "out"
    cfg.data_dir = str(out).encode()
    mesh = Mesh(cfg)
    g = golden("cfg1_l5")
    with Model(cfg) as m:
        m.initial_temperature()
        for s in range(4):
            m.step(write_output=True)
        m.output_wait()
    # a step's output is taken after its Stokes solve and before update_temperature
    # (Main.c:61-63): the temperature the step started from, its velocity and stress
    for s in range(4):
        assert sorted(os.listdir(out / f"{s:07d}")) == sorted(f"{n}.0.{s:07d}" for n in NAMES)
        got_T = np.loadtxt(out / f"{s:07d}/temperature.0.{s:07d}")
        np.testing.assert_allclose(got_T, g[f"step{s:04d}/T"], rtol=1e-6, atol=1e-12)
        got_V = np.loadtxt(out / f"{s:07d}/velocity.0.{s:07d}")
        np.testing.assert_allclose(got_V[:, 0], g[f"step{s:04d}/V0"], rtol=1e-5, atol=1e-9)
        np.testing.assert_allclose(got_V[:, 1], g[f"step{s:04d}/V1"], rtol=1e-5, atol=1e-9)
    # byte for byte against the synchronous writer on the model's own fields
    with Model(cfg) as m:
        m.initial_temperature()
        m.buoyancy_force()
        m.viscosity()
        m.velocity_pressure_KGF_matrix()
        m.solve_velocity_pressure()
        d = tmp_path / "async"
        m.output_async(str(d), 0)
        m.output_wait()
        _same_as_sync_writer(mesh, tmp_path, 0, _fields(m), d)


def test_outputs_in_flight_while_stepping(tmp_path):
    cfg = Config.from_input(golden_input("hang11_l6"))
    cfg.max_citcom_cycle, cfg.max_cg_cycle = 20, 100    # a capped, quick replica step
    mesh = Mesh(cfg)
    d = tmp_path / "o"
    with Model(cfg) as m:
        m.initial_temperature()
        snaps = {}
        for s in range(3):
            m.step()
            snaps[s] = _fields(m)
            m.output_async(str(d), s, binary=True)   # three outputs queued back to back
        m.output_wait()
        for s in range(3):
            _same_as_sync_writer(mesh, tmp_path, s, snaps[s], d)
            raw = (d / f"{s:07d}/fields.0.{s:07d}.bin").read_bytes()
            assert raw[:8] == b"MCLGOUT1"
            ver, nno, nel, ts = np.frombuffer(raw[8:24], np.int32)
            assert (ver, nno, nel, ts) == (1, m.nno, m.nel, s)
            body = np.frombuffer(raw[32:], np.float64)
            X, Z, T, V0, V1 = (body[i * nno:(i + 1) * nno] for i in range(5))
            P = body[5 * nno:5 * nno + nel]
            S, vis = body[5 * nno + nel:6 * nno + nel], body[6 * nno + nel:]
            np.testing.assert_array_equal(X, mesh.get("X")[:nno])
            for name, a in (("T", T), ("V0", V0), ("V1", V1), ("P", P), ("stress", S), ("vis", vis)):
                np.testing.assert_array_equal(a, snaps[s][name], err_msg=name)


def test_write_errors_are_reported(tmp_path):
    blocker = tmp_path / "file"
    blocker.write_text("not a directory")
    cfg = Config.from_input(golden_input("cfg1_l5"))
    with Model(cfg) as m:
        m.initial_temperature()
        m.step()
        m.output_async(str(blocker / "sub"), 0)
        with pytest.raises(MclgError) as e:
            m.output_wait()
        assert e.value.status == IO_ERROR
        m.output_async(str(tmp_path / "ok"), 1)     # the writer carries on after an error
        m.output_wait()
        assert os.path.exists(tmp_path / "ok" / "0000001" / "temperature.0.0000001")
