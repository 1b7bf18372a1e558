"""The Main.c-style driver and the solver status codes, on the GPU.

- mclg_run (Main.c:3-80 over the C ABI) writes the files of Output.c:4-156
  under data_dir and prints the per-step iteration counts; they must agree
  with the reference's own files and counts for the same .input;
- iteration caps and non-finite values come back in mclg_step_stats.status
  (the reference prints and carries on, or runs on with NaN fields); the
  context stays usable afterwards.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest
from conftest import ROOT, golden, golden_input, rel
from oracle_port import Oracle

from mantle_convection_lab_gb300 import Config, Model
from mantle_convection_lab_gb300.api import CAP_REACHED, NAN, OK

pytestmark = pytest.mark.gpu

RUN = os.path.join(ROOT, "mantle_convection_lab_gb300", "mclg_run")
FIELD_TOL = 1e-8


def parse(b):
    return np.array([float(v) for v in b.decode().split()])


def test_driver_files_and_counts_match_reference(tmp_path):
    g = golden("cfg1_l5")
    shutil.copy(golden_input("cfg1_l5"), tmp_path / "case.input")
    p = subprocess.run([RUN, "case.input"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    uz = [int(l.split()[0]) for l in p.stdout.splitlines() if " dv = " in l]
    heat = [int(l.split()[-1]) for l in p.stdout.splitlines() if l.startswith("Temperature CG cycle")]
    want_uz = g["series/uzawa_cycles"]
    assert len(uz) == len(want_uz) and max(abs(a - int(b)) for a, b in zip(uz, want_uz)) <= 1
    # the reference prints one extra heat count first (its initial_T_dot solve)
    assert heat == [int(v) for v in g["series/heat_cg_cycles"][1:]]
    texts = sorted(k[5:] for k in g.files if k.startswith("text/"))
    produced = sorted(os.path.relpath(os.path.join(r, f), tmp_path / "out")
                      for r, _, fs in os.walk(tmp_path / "out") for f in fs)
    assert produced == texts
    for k in texts:
        want = bytes(g["text/" + k])
        got = (tmp_path / "out" / k).read_bytes()
        if "coord" in k:
            assert got == want, k
            continue
        # six significant digits in the files: compare the values they hold
        assert got.count(b"\n") == want.count(b"\n"), k
        a, b = parse(got), parse(want)
        assert rel(a, b) < 1e-6, (k, rel(a, b))


def _cfg(case, **over):
    c = Config.from_input(golden_input(case))
    for k, v in over.items():
        setattr(c, k, v)
    return c


def test_uzawa_cap_reported_and_iterate_matches_oracle():
    """max_citcom_cycle=1: the status says so, and the capped iterate is the reference algorithm's."""
    c = _cfg("cfg1_l5", max_citcom_cycle=1)
    o = Oracle(c)
    with Model(c) as m:
        m.initial_temperature()
        for s in range(2):
            st = m.step()
            so = o.step()
            assert st.status == CAP_REACHED
            assert st.uzawa_cycles == so["uzawa_cycles"] == 1
            for f in ("V0", "V1", "P", "stress", "T"):
                e = rel(m.get(f), o.get(f))
                assert e < FIELD_TOL, (s, f, e)
    o.close()


def test_converged_solver_cap_reported():
    c = _cfg("cfg1_l5", precision=1, stokes_rtol=1e-30, max_refine=2)
    with Model(c) as m:
        m.initial_temperature()
        st = m.step()
        assert st.status == CAP_REACHED and st.refine_passes == 2
        assert np.isfinite(m.get("V0")).all()


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_nan_temperature_reported(precision):
    """A NaN in T reaches the Stokes solve through buoyancy and viscosity; the
    solver stops, reports MCLG_NAN, and the context keeps working."""
    c = _cfg("cfg1_l5", precision=precision, A=1.0)
    with Model(c) as m:
        m.initial_temperature()
        T = m.get("T")
        T[m.nno // 2] = np.nan
        m.set("T", T)
        st = m.step()
        assert st.status == NAN
        m.initial_temperature()
        st = m.step()
        assert st.status in (OK, CAP_REACHED)
        assert np.isfinite(m.get("V0")).all() and np.isfinite(m.get("T")).all()
