"""The converged Stokes solver on refined meshes (precision mixed / fp64mg with
hanging nodes, k_qt.cu), checked independently of its own residual:

- the solution satisfies the hanging-node relations (x_h = mean of its two
  parents, Connection.c:59-276) and the conforming system
  C^T (F - K d - G p) = 0, G^T d = 0 to the solver's tolerance, evaluated here
  in numpy with the reference's own assembled K, G and F (the fixtures'
  CSR dumps) and a constraint matrix built from the mesh's hanging list;
- it equals a direct sparse solve of that system (scipy);
- FP32 inner solves (mixed) reach the same FP64 residual as fp64mg;
- a remeshed |grad T| mesh with chained hanging nodes solves over several
  steps.
"""
import numpy as np
import pytest
from conftest import golden, golden_input, rel

from mantle_convection_lab_gb300 import Config, Model, amr

pytestmark = pytest.mark.gpu


def constraint_matrix(m, neq):
    """C (neq x neq, scipy) with d = C d: the identity on every equation except a
    hanging node's, whose row averages its parents' rows (chains resolved)."""
    sp = pytest.importorskip("scipy.sparse")
    node = m.mesh("node")
    idv = m.mesh("id").reshape(2, -1)
    hang = m.mesh("hang").reshape(3, -1)
    at = {int(g): i for i, g in enumerate(node)}
    parents = {at[int(h)]: (at[int(a)], at[int(b)]) for h, a, b in hang.T}

    def expand(A, c, w, out):
        eq = idv[c, A]
        if eq < 0:
            return
        if A in parents:
            for P in parents[A]:
                expand(P, c, 0.5 * w, out)
        else:
            out[eq] = out.get(eq, 0.0) + w

    rows, cols, vals = [], [], []
    for A in range(node.size):
        for c in range(2):
            eq = idv[c, A]
            if eq < 0:
                continue
            terms = {}
            if A in parents:
                for P in parents[A]:
                    expand(P, c, 0.5, terms)
            else:
                terms[eq] = 1.0
            for k, w in terms.items():
                rows.append(eq)
                cols.append(k)
                vals.append(w)
    C = sp.csr_matrix((vals, (rows, cols)), shape=(neq, neq))
    reduced = np.array(sorted({eq for A in range(node.size) for c in range(2)
                               if (eq := idv[c, A]) >= 0 and A not in parents}), np.int64)
    return C, reduced


def csr(g, name, lev, shape):
    sp = pytest.importorskip("scipy.sparse")
    return sp.csr_matrix((g[f"ops/{name}_val@{lev}"], g[f"ops/{name}_col@{lev}"], g[f"ops/{name}_ptr@{lev}"]),
                         shape=shape)


def _cfg(case, precision):
    c = Config.from_input(golden_input(case))
    c.precision = precision
    c.warm_start = 0
    c.stokes_rtol = 1e-9
    c.max_refine, c.max_outer = 40, 2000
    return c


@pytest.mark.parametrize("case,precision", [("hang11_l6", 2), ("hang11_l6", 1), ("dev12_l7", 1), ("hang11v_l6", 1)])
def test_conforming_residual_and_constraints(case, precision):
    g = golden(case)
    with Model(_cfg(case, precision)) as m:
        lev = m.max_level - 1
        m.initial_temperature()
        m.buoyancy_force()
        m.viscosity()
        m.velocity_pressure_KGF_matrix()
        st = m.solve_velocity_pressure()
        assert st.status == 0, st.status
        d, p = m.get("d"), m.get("P")
        neq, nel = d.size, p.size
        C, reduced = constraint_matrix(m, neq)
        K = csr(g, "K", lev, (neq, neq))
        G = csr(g, "G", lev, (neq, nel))
        F = g[f"ops/F@{lev}"]
        assert m.nh > 0
        # hanging relations hold on the returned d
        assert np.abs(C @ d - d).max() <= 1e-14 * np.abs(d).max()
        Rm = C.T @ (F - K @ d - G @ p)
        Rc = G.T @ d
        fn = np.linalg.norm(C.T @ F)
        res = np.sqrt(np.linalg.norm(Rm) ** 2 + np.linalg.norm(Rc) ** 2) / fn
        assert res < 2e-9, (res, st.res_momentum, st.res_continuity, st.refine_passes)
        print(case, precision, "refine", st.refine_passes, "minres", st.uzawa_cycles, "res", res)


def test_equals_direct_solve():
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    case = "hang11_l6"
    g = golden(case)
    with Model(_cfg(case, 2)) as m:
        lev = m.max_level - 1
        m.initial_temperature()
        m.step()
        d, p = m.get("d"), m.get("P")
        neq, nel = d.size, p.size
        C, reduced = constraint_matrix(m, neq)
        K = csr(g, "K", lev, (neq, neq))
        G = csr(g, "G", lev, (neq, nel))
        F = g[f"ops/F@{lev}"]
    Cr = C[:, reduced]
    A = sp.bmat([[Cr.T @ K @ Cr, Cr.T @ G], [G.T @ Cr, None]]).tocsc()
    # pressure is unique up to the null modes of G: fix it by a tiny regularisation
    A = A + sp.diags(np.r_[np.zeros(reduced.size), 1e-12 * np.ones(nel)])
    x = spla.spsolve(A, np.r_[Cr.T @ F, np.zeros(nel)])
    d_ref = Cr @ x[:reduced.size]
    assert rel(d, d_ref) < 1e-7
    # the pressure is determined up to the null space of C^T G (larger than G's on a
    # refined mesh): compare what the momentum equation sees
    assert rel(Cr.T @ (G @ p), Cr.T @ (G @ x[reduced.size:])) < 1e-6


def test_remeshed_mesh_steps_converge():
    cfg = Config.from_input(amr.CFG2_INPUT)
    cfg.level = 9
    cfg.precision = 1
    cfg.warm_start = 3
    cfg.stokes_rtol = 1e-8
    with Model(cfg, leaves=amr.uniform_leaves(cfg.level - 1, 6)) as m:
        m.initial_temperature()
        m.remesh(0.2, 6, 8)
        assert m.nh > 0
        for s in range(4):
            st = m.step()
            assert st.status == 0 and st.res_momentum < 1e-8 and st.res_continuity < 1e-8, (s, st.status,
                                                                                         st.res_momentum)
            assert np.isfinite(m.get("T")).all()
        print("remeshed", m.nel, "elements", m.nh, "hanging; last step", st.refine_passes, "passes",
              st.uzawa_cycles, "MINRES iterations")
