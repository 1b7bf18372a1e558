"""Multigrid transfer maps of the reference's solver="mg", restated in Python
-- TEST INFRASTRUCTURE ONLY (tests/ use it as the checker of the engine's own
map builder; the product never imports it).

Inputs are one rank's mesh arrays of two consecutive levels, as the host mesh
API returns them: node (sorted global node ids), ien (a-major global ids),
id (d-major equation numbers, -1 fixed), Mcode (level in the low 4 bits).

    interp(lo, up, lev_lo) -> (n[neq_up], src[4, neq_up])
        build_interp_conn, Connection.c:708-930 (the local part, one rank)
    project(lo, up) -> up_eq[neq_lo]
        build_project_conn, Connection.c:1051-1210, and the local table of
        setup_project_comm_frame, Connection.c:1211-1251
"""
import numpy as np


def _index(node):
    return {int(g): i for i, g in enumerate(node)}


def interp(lo, up, lev_lo):
    nlo, nup = len(lo["node"]), len(up["node"])
    nel = len(lo["Mcode"])
    ien = lo["ien"].reshape(4, nel)
    id_lo = lo["id"].reshape(2, nlo)
    id_up = up["id"].reshape(2, nup)
    neq = int((id_up >= 0).sum())
    at_lo, at_up = _index(lo["node"]), _index(up["node"])
    n = np.zeros(neq, np.int32)
    src = np.full((4, neq), -1, np.int32)
    check = np.zeros(nup, bool)
    for e in range(nel):
        if (int(lo["Mcode"][e]) & 15) > lev_lo:        # Connection.c:753-754
            continue
        for p in range(4):                              # :756-782, edge midpoints
            n1, n2 = int(ien[p, e]), int(ien[(p + 1) % 4, e])
            j = at_up.get((n1 + n2) // 2, -1)
            if j < 0 or check[j]:
                continue
            check[j] = True
            i1, i2 = at_lo[n1], at_lo[n2]
            for d in range(2):
                eu = id_up[d, j]
                if eu >= 0:
                    src[0, eu] = id_lo[d, i1]
                    src[1, eu] = id_lo[d, i2]
                    n[eu] = 2
        c = sum(int(ien[p, e]) for p in range(4)) // 4   # :826-845, element centre
        j = at_up.get(c, -1)
        if j < 0 or check[j]:
            continue
        check[j] = True
        for d in range(2):
            eu = id_up[d, j]
            if eu >= 0:
                for p in range(4):
                    src[p, eu] = id_lo[d, at_lo[int(ien[p, e])]]
                n[eu] = 4
    for i in range(nlo):                                # :890-930, shared nodes
        j = at_up.get(int(lo["node"][i]), -1)
        if j < 0 or check[j]:
            continue
        check[j] = True
        for d in range(2):
            eu = id_up[d, j]
            if eu >= 0:
                src[n[eu], eu] = id_lo[d, i]
                n[eu] += 1
    return n, src


def project(lo, up):
    nlo, nup = len(lo["node"]), len(up["node"])
    id_lo = lo["id"].reshape(2, nlo)
    id_up = up["id"].reshape(2, nup)
    neq = int((id_lo >= 0).sum())
    at_lo = _index(lo["node"])
    up_eq = np.full(neq, -1, np.int32)
    for i in range(nup):                                # Connection.c:1095-1113
        j = at_lo.get(int(up["node"][i]), -1)
        if j < 0:
            continue
        for d in range(2):
            el = id_lo[d, j]
            if el >= 0:
                up_eq[el] = id_up[d, i]
    return up_eq


def level_arrays(mesh, lev):
    """The arrays interp/project read, from an engine Mesh (api.Mesh)."""
    return {k: mesh.get(k, lev) for k in ("node", "ien", "id", "Mcode")}
