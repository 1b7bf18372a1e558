"""Host side of the C ABI, without a GPU.

- every function that include/mclg.h declares is exported by libmclg.so;
- the .input reader follows the getpar rules of Parsing.c:54-141 (blanks,
  comments, quoting, several pairs per line, last occurrence wins) and the
  defaults of Input.c:3-99;
- errors come back as status codes (the reference exits instead);
- the Output.c writer reproduces the reference's own text files byte for byte
  when given the reference's fields.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest
from conftest import ROOT, golden, golden_input

from mantle_convection_lab_gb300 import Config, MclgError, Mesh, api

HEADER = os.path.join(ROOT, "include", "mclg.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mclg_\w+)\s*\(", text)))


def test_every_declared_function_is_exported():
    names = declared_functions()
    assert len(names) >= 30
    L = C.CDLL(api.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_struct_layouts_and_status_strings():
    L = api.lib()   # raises if the ctypes layouts differ from the library's
    assert L.mclg_config_sizeof() == C.sizeof(Config)
    strings = {L.mclg_status_string(s).decode() for s in range(8)}
    assert len(strings) == 8 and "unknown status" not in strings
    assert L.mclg_status_string(99).decode() == "unknown status"


def write(tmp_path, text, name="case.input"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_defaults_follow_input_c(tmp_path):
    c = Config.from_input(write(tmp_path, "# nothing but a comment\n\n"))
    assert c.data_dir == b"." and c.solver == b"jc"
    assert (c.level, c.mg_min_level, c.nprox, c.nproz) == (1, 1, 2, 2)
    assert (c.model_length, c.model_height) == (2.0, 1.0)
    assert bytes(c.top_v_bc[:2]) == b"sv" and bytes(c.lef_v_bc[:2]) == b"vs"
    assert list(c.top_v_bc_val) == [0.0, 0.0]
    assert (c.top_T_bc, c.bot_T_bc, c.lef_T_bc, c.rig_T_bc) == (b"T", b"T", b"F", b"F")
    assert (c.top_T_bc_val, c.bot_T_bc_val) == (0.0, 1.0)
    assert (c.T_ini, c.T_mantle, c.T_mantle_perturb, c.T_wave_number) == (1, 0.5, 0.01, 6)
    assert (c.Rayleigh, c.A, c.refT, c.lower_mantle_jump) == (1e7, 0.0, 0.5, 1.0)
    assert (c.max_timestep, c.save_spacing, c.Q, c.theta) == (0, 1, 0.0, 0.0)
    assert (c.cg_precondition, c.accuracy, c.citcom_solver_accu) == (0, 0.001, 0.001)
    assert (c.develop_mode, c.max_citcom_cycle, c.max_cg_cycle, c.zero_P) == (1, 375, 200, 1)
    assert c.precision == 0 and c.warm_start == 0
    assert (c.grain_damage, c.lowest_vis, c.highest_vis) == (0, 1.0, 1.0)     # Input.c:58-59, 95
    assert (c.mg_smoother, c.mg_cheb_lmax, c.mg_cheb_ratio) == (0, 2.5, 4.0)  # engine's own options
    assert c.mg_fine_levels == 2
    c = Config.from_input(write(tmp_path, "mg_smoother=1\nmg_cheb_lmax=2.2\nmg_cheb_ratio=5\n"))
    assert (c.mg_smoother, c.mg_cheb_lmax, c.mg_cheb_ratio) == (1, 2.2, 5.0)


def test_getpar_tokenisation(tmp_path):
    text = (
        "   level=6 mg_min_level=2\tnprox=1   # trailing comment level=9\n"
        "# level=8\n"
        "data_dir=\"./with space\" solver='cg'\n"
        "Rayleigh=1e5\n"
        "Rayleigh=2.5e6\n"                  # the last occurrence wins
        "top_v_bc=VSX bot_T_bc=Fixed\n"     # v_bc keeps two characters, T_bc one
        "top_v_bc_val=1.5\n"                # a short vector leaves the rest as it was
        "bot_v_bc_val=0.25,-3\n"
        "precision=mixed stokes_rtol=1e-9 warm_start=1\n"
        "ic_seed=18446744073709551615\n"
    )
    c = Config.from_input(write(tmp_path, text))
    assert (c.level, c.mg_min_level, c.nprox) == (6, 2, 1)
    assert c.data_dir == b"./with space" and c.solver == b"cg"
    assert c.Rayleigh == 2.5e6
    assert bytes(c.top_v_bc[:2]) == b"VS" and c.bot_T_bc == b"F"
    assert list(c.top_v_bc_val) == [1.5, 0.0]
    assert list(c.bot_v_bc_val) == [0.25, -3.0]
    assert c.precision == 1 and c.stokes_rtol == 1e-9 and c.warm_start == 1
    assert c.ic_seed == 2**64 - 1
    assert Config.from_input(write(tmp_path, "precision=fp64mg\n", "b.input")).precision == 2
    assert Config.from_input(write(tmp_path, "precision=other\n", "c.input")).precision == 0


def test_fixture_inputs_parse_as_the_reference_read_them():
    c = Config.from_input(golden_input("cfg1_l5"))
    assert (c.level, c.mg_min_level, c.max_timestep, c.cg_precondition) == (5, 3, 3, 1)
    assert c.accuracy == 1e-20 and c.citcom_solver_accu == 1e-8 and c.theta == 0.5
    assert bytes(c.top_v_bc[:2]) == b"SV" and bytes(c.lef_v_bc[:2]) == b"VS"
    assert c.data_dir == b"./out" and c.T_ini == -2 and c.ic_seed == 42


def test_missing_input_file_is_an_io_error(tmp_path):
    with pytest.raises(MclgError) as e:
        Config.from_input(str(tmp_path / "absent.input"))
    assert e.value.status == api.IO_ERROR


@pytest.mark.parametrize("extra,needle", [
    ("nprox=2\nnproz=1\n", "nprox"),
    ("level=3\nmg_min_level=3\n", "mg_min_level"),
    ("level=20\nmg_min_level=1\n", "level"),
    ("level=4\nmg_min_level=1\ndevelop_mode=99\n", "develop_mode"),
])
def test_mesh_rejects_bad_inputs(tmp_path, extra, needle):
    c = Config.from_input(write(tmp_path, "nprox=1\nnproz=1\nlevel=4\nmg_min_level=1\ndevelop_mode=0\n" + extra))
    with pytest.raises(MclgError) as e:
        Mesh(c)
    assert e.value.status == api.BAD_INPUT
    assert needle in str(e.value)


def test_mesh_buffer_checks(tmp_path):
    c = Config.from_input(write(tmp_path, "nprox=1\nnproz=1\nlevel=4\nmg_min_level=1\ndevelop_mode=0\n"))
    m = Mesh(c)
    L = api.lib()
    out = np.zeros(3, np.int32)
    assert L.mclg_mesh_get(m._h, api.MESH["node"], -1, api._iptr(out), 3) == api.BAD_INPUT
    assert b"buffer has 3" in L.mclg_last_error()
    assert L.mclg_mesh_get(m._h, api.MESH["node"], 7, api._iptr(out), 3) == api.BAD_INPUT
    assert L.mclg_mesh_get(m._h, 99, -1, api._iptr(out), 3) == api.BAD_INPUT
    T = np.zeros(5)
    assert L.mclg_mesh_initial_temperature(m._h, -1, api._dptr(T), 5) == api.BAD_INPUT
    bad_ini = Config.from_input(write(tmp_path, "nprox=1\nnproz=1\nlevel=4\nmg_min_level=1\nT_ini=7\n", "t.input"))
    with pytest.raises(MclgError) as e:
        Mesh(bad_ini).initial_temperature()
    assert e.value.status == api.BAD_INPUT and "T_ini" in str(e.value)


def test_create_without_device_reports_no_device():
    """On a machine without a GPU, mclg_create fails with MCLG_NO_DEVICE."""
    L = api.lib()
    c = Config.from_input(golden_input("cfg1_l5"))
    h = C.c_void_p()
    rc = L.mclg_create(C.byref(h), C.byref(c))
    if rc == api.OK:
        L.mclg_destroy(h)
        pytest.skip("a CUDA device is visible")
    assert rc == api.NO_DEVICE, L.mclg_last_error()
    assert not h


def test_create_rejects_unsupported_options(tmp_path):
    L = api.lib()
    for extra, needle in (("lg_mul=1\n", b"lg_mul"), ('solver="sor"\n', b"solver")):
        c = Config.from_input(write(tmp_path, open(golden_input("cfg1_l5")).read() + extra))
        h = C.c_void_p()
        assert L.mclg_create(C.byref(h), C.byref(c)) == api.BAD_INPUT
        assert needle in L.mclg_last_error()


def test_grain_damage_is_accepted_only_where_the_reference_defines_it(tmp_path):
    """grain_damage=1 runs on a single-level mesh with the FP64 replica and solver cg or
    jc (the reference evolves only the first level its viscosity() visits); elsewhere
    it is rejected before any device work.  The accepted case gets as far as the
    device check."""
    L = api.lib()
    base = open(golden_input("gd_l5")).read()
    for extra in ("mg_min_level=3\n", 'solver="gs"\n', "precision=\"mixed\"\n", "grain_damage=2\n"):
        c = Config.from_input(write(tmp_path, base + extra))
        h = C.c_void_p()
        assert L.mclg_create(C.byref(h), C.byref(c)) == api.BAD_INPUT, extra
        assert b"grain_damage" in L.mclg_last_error()
    c = Config.from_input(golden_input("gd_l5"))
    h = C.c_void_p()
    rc = L.mclg_create(C.byref(h), C.byref(c))
    if rc == api.OK:
        L.mclg_destroy(h)
        pytest.skip("a CUDA device is visible")
    assert rc == api.NO_DEVICE, L.mclg_last_error()


@pytest.mark.parametrize("step", [0, 1, 2, 3])
def test_output_text_matches_reference_files(tmp_path, step):
    """Output.c:4-156: same file names and the same bytes, from the reference's fields."""
    g = golden("cfg1_l5")
    m = Mesh(Config.from_input(golden_input("cfg1_l5")))
    f = {k: g[f"step{step:04d}/{k}"] for k in ("T", "V0", "V1", "stress", "vis")}
    m.write_output(str(tmp_path), step, f["T"], f["V0"], f["V1"], f["stress"], f["vis"])
    names = ("coord", "temperature", "stress", "viscosity", "velocity")
    for name in names:
        rel_path = f"{step:07d}/{name}.0.{step:07d}"
        want = bytes(g["text/" + rel_path])
        got = (tmp_path / rel_path).read_bytes()
        assert got == want, (name, got[:200], want[:200])
    assert sorted(os.listdir(tmp_path / f"{step:07d}")) == sorted(f"{n}.0.{step:07d}" for n in names)


def test_output_rejects_wrong_lengths(tmp_path):
    m = Mesh(Config.from_input(golden_input("cfg1_l5")))
    z = np.zeros(m.nno - 1)
    with pytest.raises(MclgError) as e:
        m.write_output(str(tmp_path), 0, z, z, z, z, z)
    assert e.value.status == api.BAD_INPUT


def test_cnn_create_without_device_reports_no_device():
    L = api.lib()
    h = C.c_void_p()
    rc = L.mclg_cnn_create(C.byref(h), 8, 32, 6, 3, 0)
    if rc == api.OK:
        L.mclg_cnn_destroy(h)
        pytest.skip("a CUDA device is visible")
    assert rc == api.NO_DEVICE
    assert L.mclg_cnn_create(C.byref(h), 8, 32, 1, 3, 0) == api.BAD_INPUT   # depth < 2
    assert L.mclg_cnn_load(C.byref(h), b"/nonexistent/net.bin") == api.IO_ERROR


def test_restart_reads_the_file_before_the_device(tmp_path):
    """mclg_restart checks the checkpoint file before it touches a device."""
    L = api.lib()
    c = Config.from_input(golden_input("cfg1_l5"))
    h = C.c_void_p()
    assert L.mclg_restart(C.byref(h), C.byref(c), str(tmp_path / "none.ckp").encode()) == api.IO_ERROR
    junk = tmp_path / "junk.ckp"
    junk.write_bytes(b"not a checkpoint" * 8)
    assert L.mclg_restart(C.byref(h), C.byref(c), str(junk).encode()) == api.BAD_INPUT
    assert not h
