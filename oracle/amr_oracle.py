"""CPU oracle of the |grad T| refinement -- test infrastructure only.

The reference has no runtime refinement; this restates, in numpy, what the
library's refinement does so that it can be checked bit for bit:
- flags (mantle_convection_lab_gb300/csrc/cuda/k_amr.cu): |grad T| at each
  finest-level element's centre from its corner temperatures,
      dT/dx = ((T3 + T2) - (T0 + T1)) / (4 hx),  dT/dz = ((T1 + T2) - (T0 + T3)) / (4 hz),
  hx = dx_dxi = 0.5 * length / 2^level (Mesh.c:396-428), flagged when above
  frac * max (IEEE double arithmetic in the same order);
- the tree (csrc/host/mclg_amr.c): fine cells under flagged leaves ask for
  target_level, the rest for base_level; split top-down from the base grid
  while a cell below asks for more; 2:1 balance over the 8 neighbours of every
  fine cell; leaves listed by Morton start code;
- the transfer: bilinear interpolation of nodal T inside the old leaf that
  contains each new node.
"""
import numpy as np


def demorton(code):
    x = z = 0
    for i in range(16):
        x |= ((code >> (2 * i + 1)) & 1) << i
        z |= ((code >> (2 * i)) & 1) << i
    return x, z


def local_ien(mesh):
    node = mesh.get("node")
    return np.searchsorted(node, mesh.get("ien").reshape(4, -1))


def flags(mesh, T, frac):
    """Flags and |grad T| per finest-level element of a host mesh (Mesh)."""
    ienl = local_ien(mesh)
    lev = (mesh.get("Mcode") & 15).astype(np.float64)
    hx = 0.5 * (mesh.config.model_length / 2.0 ** lev)
    hz = 0.5 * (mesh.config.model_height / 2.0 ** lev)
    t0, t1, t2, t3 = (T[ienl[a]] for a in range(4))
    gx = ((t3 + t2) - (t0 + t1)) / (4.0 * hx)
    gz = ((t1 + t2) - (t0 + t3)) / (4.0 * hz)
    g = np.sqrt(gx * gx + gz * gz)
    return (g > frac * g.max()).astype(np.uint8), g


def build_leaves(mcode, flg, F, base, target):
    """Leaves (finest-level Morton start codes) of the refined tree, and the
    level map of the fine cells."""
    NF = 1 << F
    tgt = np.full((NF, NF), base, np.int32)
    for e in np.nonzero(flg)[0]:
        lvl, loc = int(mcode[e]) & 15, int(mcode[e]) >> 4
        x0, z0 = demorton(loc)
        s = 1 << (F - lvl)
        tgt[x0:x0 + s, z0:z0 + s] = target
    lv = np.zeros((NF, NF), np.int32)

    def split(l, x, z):
        s = 1 << (F - l)
        if l < target and tgt[x * s:(x + 1) * s, z * s:(z + 1) * s].max() > l:
            for i in (0, 1):
                for j in (0, 1):
                    split(l + 1, 2 * x + i, 2 * z + j)
        else:
            lv[x * s:(x + 1) * s, z * s:(z + 1) * s] = l

    nb = 1 << base
    for x in range(nb):
        for z in range(nb):
            split(base, x, z)
    while True:
        p = np.pad(lv, 1, constant_values=-1)
        nbmax = np.max([p[1 + dx:1 + dx + NF, 1 + dz:1 + dz + NF]
                        for dx in (-1, 0, 1) for dz in (-1, 0, 1)], axis=0)
        need = nbmax > lv + 1
        if not need.any():
            break
        marks = {}
        for x, z in zip(*np.nonzero(need)):
            l = int(lv[x, z])
            s = 1 << (F - l)
            marks[(x & ~(s - 1), z & ~(s - 1))] = l + 1
        for (x0, z0), nl in marks.items():
            s = 1 << (F - nl + 1)
            lv[x0:x0 + s, z0:z0 + s] = nl
    out, code = [], 0
    while code < NF * NF:
        x, z = demorton(code)
        out.append(code)
        code += 1 << (2 * (F - int(lv[x, z])))
    return np.array(out, np.int32), lv


def transfer(mesh_from, T, mesh_to):
    """Bilinear transfer of nodal T between two host meshes of the same box."""
    X = mesh_from.get("X").reshape(2, -1)
    ienl = local_ien(mesh_from)
    n = mesh_from.gnox - 1
    dxc = mesh_from.config.model_length / n
    dzc = mesh_from.config.model_height / n
    cell = np.zeros((n, n), np.int64)
    mcode = mesh_from.get("Mcode")
    F = mesh_from.max_level - 1
    for e in range(mcode.size):
        lvl, loc = int(mcode[e]) & 15, int(mcode[e]) >> 4
        x0, z0 = demorton(loc)
        s = 1 << (F - lvl)
        cell[x0:x0 + s, z0:z0 + s] = e
    Y = mesh_to.get("X").reshape(2, -1)
    cx = np.clip((Y[0] / dxc).astype(np.int64), 0, n - 1)
    cz = np.clip((Y[1] / dzc).astype(np.int64), 0, n - 1)
    e = cell[cx, cz]
    n0, n1, n2, n3 = (ienl[a][e] for a in range(4))
    x0, z0 = X[0][n0], X[1][n0]
    xi = (Y[0] - x0) / (X[0][n3] - x0)
    ze = (Y[1] - z0) / (X[1][n1] - z0)
    return (1 - xi) * ((1 - ze) * T[n0] + ze * T[n1]) + xi * (ze * T[n2] + (1 - ze) * T[n3])
