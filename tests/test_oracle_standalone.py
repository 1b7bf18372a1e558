"""The oracle's standalone input reader and uniform mesh (oracle/mesh_oracle.py)
against the reference's own dumps and the engine's builder.

bench.py's CPU baseline runs the oracle on these arrays so that it loads
nothing of the engine; they must be the reference's arrays bit for bit."""
import glob
import os

import numpy as np
import pytest
from conftest import GOLDEN, ROOT, golden, golden_input, rel

import mesh_oracle
import oracle_port
from mantle_convection_lab_gb300 import Config, Mesh

INPUTS = sorted(glob.glob(os.path.join(GOLDEN, "*.input"))) + sorted(
    glob.glob(os.path.join(ROOT, "mantle_convection_lab_gb300", "configs", "*.input")))
KEYS = list(mesh_oracle.InputConfig.INTS) + list(mesh_oracle.InputConfig.FLOATS) + ["ic_seed"]


@pytest.mark.parametrize("path", INPUTS, ids=os.path.basename)
def test_input_keys_equal_engine_parser(path):
    a, b = mesh_oracle.read_input(path), Config.from_input(path)
    for k in KEYS:
        assert getattr(a, k) == getattr(b, k), k
    for k in mesh_oracle.InputConfig.VBC:
        assert a.__dict__[k] == bytes(getattr(b, k)), k
        assert list(getattr(a, k + "_val")) == list(getattr(b, k + "_val")), k
    for k in mesh_oracle.InputConfig.TBC:
        assert a.__dict__[k] == getattr(b, k), k
    assert a.solver == bytes(b.solver)


@pytest.mark.parametrize("case", ["cfg1_l5", "cfg1_l7"])
def test_uniform_mesh_equals_reference_dump(case):
    g = golden(case)
    m = mesh_oracle.UniformMesh(mesh_oracle.read_input(golden_input(case)))
    lev = m.max_level - 1
    for k in ("Mcode", "node", "ien"):
        assert np.array_equal(m.get(k), g[f"mesh/{k}@{lev}"]), k
    X = m.get("X").reshape(2, -1)
    assert np.array_equal(X[0], g[f"mesh/X0@{lev}"]) and np.array_equal(X[1], g[f"mesh/X1@{lev}"])
    assert np.array_equal(m.get("T_bc"), g[f"mesh/T_bc@{lev}"].astype(np.int32))
    assert np.array_equal(m.get("T_bc_val"), g[f"mesh/T_bc_val@{lev}"])
    vbc = m.get("v_bc").reshape(2, -1)
    assert np.array_equal(vbc[0], g[f"mesh/v_bc0@{lev}"].astype(np.int32))
    assert np.array_equal(vbc[1], g[f"mesh/v_bc1@{lev}"].astype(np.int32))
    vv = m.get("v_bc_val").reshape(2, -1)
    assert np.array_equal(vv[0], g[f"mesh/v_bc_val0@{lev}"])
    assert np.array_equal(vv[1], g[f"mesh/v_bc_val1@{lev}"])
    assert np.array_equal(m.initial_temperature(), g[f"ops/T@{lev}"])


@pytest.mark.parametrize("name", ["cfg3_mg_1024", "cfg1_plain_64"])
def test_uniform_mesh_equals_engine_builder(name):
    """The benchmark inputs (1024^2 for configuration 3) against the engine's
    host builder, which is pinned to the reference on every fixture."""
    path = os.path.join(ROOT, "mantle_convection_lab_gb300", "configs", f"{name}.input")
    a = mesh_oracle.UniformMesh(mesh_oracle.read_input(path))
    b = Mesh(Config.from_input(path))
    lev = b.max_level - 1
    assert (a.gnox, a.gnoz, a.max_level) == (b.gnox, b.gnoz, b.max_level)
    for k in ("Mcode", "node", "ien", "v_bc", "T_bc", "X", "v_bc_val", "T_bc_val"):
        assert np.array_equal(a.get(k), b.get(k, lev)), k
    assert np.array_equal(a.initial_temperature(), b.initial_temperature())


def test_standalone_oracle_steps_equal_reference():
    g = golden("cfg1_l5")
    o = oracle_port.Oracle(golden_input("cfg1_l5"), standalone=True)
    for s in range(2):
        st = o.step()
        assert st["uzawa_cycles"] == g["series/uzawa_cycles"][s]
        for k, kk in (("V0", "V0"), ("V1", "V1"), ("P", "p"), ("d", "d")):
            assert rel(o.get(k), g[f"step{s:04d}/{kk}"]) < 1e-12, (s, k)
        assert rel(o.get("T"), g[f"heat{s:04d}/T"]) < 1e-12
    o.close()
