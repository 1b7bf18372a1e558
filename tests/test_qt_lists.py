"""The refined-mesh solver's host lists (csrc/host/mclg_qtmg.c), checked without
a GPU through what they are for.  On every level the contribution lists
assemble C^T K C: for a random K with the mesh's node-block sparsity, the
lists' sums equal C^T K C formed with scipy, C built here independently from
the mesh's hanging-node list (a hanging node's free component is the mean of its
two parents', chains followed, fixed dofs 0; Connection.c:59-276).  Meshes: the
develop_mode 11 fixture mesh (hanging nodes along the bands), and a graded mesh
whose finest level is large enough for the lists to be built in row chunks on
threads."""
import numpy as np
import pytest
from conftest import golden_input

from mantle_convection_lab_gb300 import Config, Mesh
from mantle_convection_lab_gb300.api import NB_WIDTH

sp = pytest.importorskip("scipy.sparse")


def expansion(m, lev):
    """(C over dofs 2*node + c, kind) with C[dof, reduced dof]."""
    node = m.get("node", lev)
    nno = node.size
    vbc = m.get("v_bc", lev).reshape(2, nno)
    hang = m.get("hang", lev).reshape(3, -1)
    at = {int(g): i for i, g in enumerate(node)}
    parents = {at[int(h)]: (at[int(a)], at[int(b)]) for h, a, b in hang.T}
    fixed = vbc == ord("V")
    kind = np.zeros(2 * nno, np.int32)
    for A in range(nno):
        for c in range(2):
            kind[2 * A + c] = 0 if fixed[c, A] else (2 if A in parents else 1)
    red = np.flatnonzero(kind == 1)
    col = np.full(2 * nno, -1)
    col[red] = np.arange(red.size)

    def expand(A, c, w, out):
        if fixed[c, A]:
            return
        if A in parents:
            for P in parents[A]:
                expand(P, c, 0.5 * w, out)
        else:
            out[2 * A + c] = out.get(2 * A + c, 0.0) + w

    rows, cols, vals = [], [], []
    for d in np.flatnonzero(kind > 0):
        terms = {}
        expand(int(d) >> 1, int(d) & 1, 1.0, terms)
        for r, w in terms.items():
            rows.append(d)
            cols.append(col[r])
            vals.append(w)
    return sp.csr_matrix((vals, (rows, cols)), shape=(2 * nno, red.size)), kind, col


def check_level(m, lev, seed):
    q = m.qt(lev)
    nno = q["nno"]
    C, kind, col = expansion(m, lev)
    np.testing.assert_array_equal(q["kind"], kind)
    # a random node-block K on the mesh's sparsity: K64[(k*nno + A)*4 + 2c + c'] couples
    # (A, c) with (the k-th neighbour of A, c')
    nb = m.get("nb", lev).reshape(nno, NB_WIDTH)
    cnt = (nb >= 0).sum(1)
    width = int(cnt.max())
    rng = np.random.default_rng(seed)
    K64 = rng.standard_normal((width, nno, 4))
    K64[np.arange(width)[:, None] >= cnt[None, :]] = 0.0
    A_, k_ = np.nonzero((np.arange(width)[None, :] < cnt[:, None]))
    B_ = nb[A_, k_]
    r, cidx, v = [], [], []
    for cc in range(4):
        r.append(2 * A_ + (cc >> 1))
        cidx.append(2 * B_ + (cc & 1))
        v.append(K64[k_, A_, cc])
    K = sp.csr_matrix((np.concatenate(v), (np.concatenate(r), np.concatenate(cidx))), shape=(2 * nno, 2 * nno))
    want = (C.T @ K @ C).tocsr()
    # the lists' sums
    flat = K64.ravel()
    row_node = np.repeat(np.arange(nno), np.diff(q["rc_off"]))
    slot, cc = q["rc_tgt"] >> 2, q["rc_tgt"] & 3
    assert (slot < q["rcnt"][row_node]).all()
    B = q["rnb"][slot * nno + row_node]
    rd, cd = 2 * row_node + (cc >> 1), 2 * B + (cc & 1)
    assert (kind[rd] == 1).all() and (kind[cd] == 1).all()
    got = sp.csr_matrix((q["rc_w"] * flat[q["rc_src"]], (col[rd], col[cd])), shape=want.shape)
    diff = abs(got - want).max() if want.nnz else 0.0
    assert diff <= 1e-13 * abs(want).max(), (lev, diff)
    # every column of a row is listed once, ascending
    for A in range(0, nno, max(1, nno // 64)):
        cols_A = q["rnb"][np.arange(q["rcnt"][A]) * nno + A]
        assert (np.diff(cols_A) > 0).all()
    return q


def test_lists_on_the_hanging_band_mesh():
    m = Mesh(Config.from_input(golden_input("hang11_l6")))
    for lev in range(m.max_level - 1, 3, -1):
        check_level(m, lev, lev)


def test_lists_on_a_graded_mesh_built_in_chunks():
    c = Config.from_input(golden_input("cfg1_l5"))
    c.level, c.mg_min_level, c.develop_mode = 10, 7, 0
    base = Mesh(c, leaves=np.arange(0, 1 << 18, 1 << 6, dtype=np.int32))     # 64 x 64 base in 512 x 512
    flags = (np.random.default_rng(9).random(base.nel) < 0.08).astype(np.uint8)
    m = Mesh(c, leaves=base.amr_leaves(flags, 6, 9))
    q = check_level(m, m.max_level - 1, 1)
    assert q["nno"] >= 2 * 8192          # more than one row chunk
    assert m.nh > 0
