"""ctypes driver of the CPU oracle (oracle/oracle.c) -- test infrastructure.

The mesh arrays (ien, node list, BC codes, hanging nodes) come from the host
mesh builder of the engine, which tests pin bit-exact against the
reference's own arrays, or -- with standalone=True, for uniform meshes --
from oracle/mesh_oracle.py, which loads nothing of the engine; everything
numerical is recomputed here on the CPU.

    r = run("case.input", steps=3)      # dict of T, V0, V1, P, d, stress, vis, stats per step
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from build_oracle import LIB, build  # noqa: E402

_L = None
GET = {"T": 0, "V0": 1, "V1": 2, "P": 3, "d": 4, "stress": 5, "vis": 6, "buoyancy": 7, "F": 8, "Kdiag": 9,
       "tau0": 10, "tau1": 11, "heat_F": 12, "gs": 13}


def lib():
    global _L
    if _L is None:
        build()
        _L = C.CDLL(LIB)
        vp = C.c_void_p
        _L.orc_new.restype = vp
        _L.orc_new.argtypes = [C.c_int] * 5 + [vp] * 8 + [C.c_int] + [vp] * 7
        for n in ("orc_free", "orc_set_T", "orc_step", "orc_stokes", "orc_assemble", "orc_kmul", "orc_gmul",
                  "orc_gtmul"):
            getattr(_L, n).restype = None
        _L.orc_free.argtypes = [vp]
        _L.orc_set_T.argtypes = [vp, vp]
        _L.orc_step.argtypes = [vp, vp]
        _L.orc_stokes.argtypes = [vp, vp]
        _L.orc_assemble.argtypes = [vp]
        _L.orc_kmul.argtypes = [vp, vp, vp]
        _L.orc_gmul.argtypes = [vp, vp, vp]
        _L.orc_gtmul.argtypes = [vp, vp, vp]
        _L.orc_get.restype = C.c_int
        _L.orc_get.argtypes = [vp, C.c_int, vp]
        _L.orc_sizes.argtypes = [vp, vp]
        _L.orc_cg_sample.restype = C.c_int
        _L.orc_cg_sample.argtypes = [vp, C.c_int]
        _L.orc_mg_attach.restype = C.c_int
        _L.orc_mg_attach.argtypes = [vp, C.c_int, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int]
        _L.orc_set_caps.restype = None
        _L.orc_set_caps.argtypes = [vp, C.c_int, C.c_int]
        _L.orc_initial_temperature.restype = None
        _L.orc_initial_temperature.argtypes = [C.c_int, vp, vp, C.c_uint64, C.c_int, vp, vp, vp]
    return _L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


SOLVERS = {b"cg": 0, b"jc": 1, b"gs": 2, b"mg": 3}


class Oracle:
    """One CPU model built from a .input file (or a Config) and the engine's host
    mesh (from develop_mode, or from a leaf list).  With solver="mg" every
    level from mg_min_level up gets its own CPU model (its K from the level's
    initial temperature, as in the reference) and the transfer maps of
    oracle/mg_oracle.py."""

    def __init__(self, cfg, threads=1, leaves=None, standalone=False, mesh_level=None):
        if standalone:
            # uniform meshes from oracle/mesh_oracle.py: the engine's library is not loaded;
            # mesh_level < cfg.level gives the uniform grid of that level (seeded T keyed by cfg.level's grid)
            import mesh_oracle
            if isinstance(cfg, (str, os.PathLike)):
                cfg = mesh_oracle.read_input(cfg)
            if leaves is not None or cfg.solver == b"mg":
                raise ValueError("the standalone oracle covers uniform meshes with the cg/jc/gs solvers")
            m = mesh_oracle.UniformMesh(cfg, level=mesh_level)
        else:
            from mantle_convection_lab_gb300.api import Config, Mesh
            if isinstance(cfg, (str, os.PathLike)):
                cfg = Config.from_input(cfg)
            m = Mesh(cfg, leaves=leaves)
        self.cfg = cfg
        self.mesh = m
        self._keep = []
        self._lv = []
        fl = m.max_level - 1
        self._o = self._level(fl, threads)
        sz = np.zeros(4, np.int32)
        lib().orc_sizes(self._o, _p(sz))
        self.nel, self.nno, self.neq, self.hneq = map(int, sz)
        if cfg.solver == b"mg":
            self._attach_mg(threads)
        self.set_T(m.initial_temperature())

    def _level(self, lev, threads):
        m, cfg, k = self.mesh, self.cfg, self._keep.append
        node = m.get("node", lev)
        nel, nno = m.get("Mcode", lev).size, node.size
        ienl = np.ascontiguousarray(np.searchsorted(node, m.get("ien", lev)), np.int32); k(ienl)
        elev = np.ascontiguousarray(m.get("Mcode", lev) & 15, np.int32); k(elev)
        node = node.astype(np.int32); k(node)
        X = m.get("X", lev); k(X)
        vbc = np.ascontiguousarray(m.get("v_bc", lev).astype(np.uint8)); k(vbc)
        vbcval = m.get("v_bc_val", lev); k(vbcval)
        tbc = np.ascontiguousarray(m.get("T_bc", lev).astype(np.uint8)); k(tbc)
        tbcval = m.get("T_bc_val", lev); k(tbcval)
        hang = m.get("hang", lev).reshape(3, -1)
        nh = hang.shape[1]
        hang = np.ascontiguousarray(np.searchsorted(node, hang), np.int32); k(hang)
        L, H = cfg.model_length, cfg.model_height
        dx = np.array([L / (1 << l) for l in range(16)]); k(dx)
        dz = np.array([H / (1 << l) for l in range(16)]); k(dz)
        dpar = np.array([cfg.Rayleigh, cfg.A, cfg.refT, cfg.lower_mantle_jump, cfg.Q, cfg.theta, cfg.accuracy,
                         cfg.citcom_solver_accu, cfg.vis_min, cfg.vis_max, cfg.lowest_vis, cfg.highest_vis]); k(dpar)
        # grain_damage: the reference evolves the grain size on the first level it visits
        # (mg_min_level); only on a single-level mesh is that the finest one
        grain = int(cfg.grain_damage == 1 and lev == m.max_level - 1 and cfg.mg_min_level == lev)
        ipar = np.array([cfg.max_citcom_cycle, cfg.max_cg_cycle, cfg.cg_precondition, cfg.check_v_only,
                         SOLVERS.get(bytes(cfg.solver), 0), cfg.zero_P, cfg.AMR, cfg.auto_accuracy, threads,
                         grain], np.int32); k(ipar)
        hp = [hang[i] if nh else np.zeros(1, np.int32) for i in range(3)]
        self._keep.extend(hp)
        if lev == m.max_level - 1:
            self.ienl, self.elev, self.node, self.X = ienl, elev, node, X
        return lib().orc_new(nel, nno, m.gnox, m.gnoz, lev, _p(ienl), _p(elev), _p(node), _p(X), _p(vbc),
                             _p(vbcval), _p(tbc), _p(tbcval), nh, _p(hp[0]), _p(hp[1]), _p(hp[2]), _p(dx),
                             _p(dz), _p(dpar), _p(ipar))

    def _attach_mg(self, threads):
        import mg_oracle
        m, cfg = self.mesh, self.cfg
        lo, fl = cfg.mg_min_level, m.max_level - 1
        arr = {lev: mg_oracle.level_arrays(m, lev) for lev in range(lo, fl + 1)}
        orcs, itp_n, itp_src, prj = [], [], [], []
        for lev in range(lo, fl + 1):
            if lev < fl:
                o = self._level(lev, threads)
                T = np.ascontiguousarray(m.initial_temperature(lev)); self._keep.append(T)
                lib().orc_set_T(o, _p(T))
                self._lv.append(o)
                orcs.append(o)
                prj.append(np.ascontiguousarray(mg_oracle.project(arr[lev], arr[lev + 1]), np.int32))
            else:
                orcs.append(self._o)
                prj.append(np.zeros(1, np.int32))
            if lev > lo:
                n, src = mg_oracle.interp(arr[lev - 1], arr[lev], lev - 1)
                itp_n.append(np.ascontiguousarray(n, np.int32))
                itp_src.append(np.ascontiguousarray(src, np.int32))
            else:
                itp_n.append(np.zeros(1, np.int32))
                itp_src.append(np.zeros(1, np.int32))
        self._keep.extend(itp_n + itp_src + prj)
        ptrs = lambda xs: (C.c_void_p * len(xs))(*[x.ctypes.data for x in xs])
        lv = (C.c_void_p * len(orcs))(*orcs)
        self._keep.append(lv)
        rc = lib().orc_mg_attach(self._o, len(orcs), lv, ptrs(itp_n), ptrs(itp_src), ptrs(prj), cfg.mg_cycle,
                                 cfg.mg_finest_iteration, cfg.mg_coarse_iteration)
        if rc != 0:
            raise ValueError("mg hierarchy needs 2..16 levels")

    def close(self):
        if self._o:
            lib().orc_free(self._o)
            self._o = None
        for o in self._lv:
            lib().orc_free(o)
        self._lv = []

    __del__ = close

    def set_T(self, T):
        self._T = np.ascontiguousarray(T, np.float64)
        lib().orc_set_T(self._o, _p(self._T))

    def step(self):
        st = np.zeros(10)
        lib().orc_step(self._o, _p(st))
        return {"uzawa_cycles": int(st[0]), "cg_cycles": int(st[1]), "heat_cg_cycles": int(st[2]),
                "dt": st[3], "model_time": st[4], "res_m": st[5], "res_c": st[6], "s_assembly": st[7],
                "s_solve": st[8], "s_heat": st[9]}

    def set_caps(self, max_citcom, max_cg):
        """max_citcom_cycle and max_cg_cycle of the following steps."""
        lib().orc_set_caps(self._o, int(max_citcom), int(max_cg))

    def stokes(self):
        st = np.zeros(10)
        lib().orc_stokes(self._o, _p(st))
        return {"uzawa_cycles": int(st[0]), "cg_cycles": int(st[1]), "res_m": st[5], "res_c": st[6]}

    def assemble(self):
        lib().orc_assemble(self._o)

    def get(self, name):
        n = {"P": self.nel, "tau0": self.nel, "tau1": self.nel, "d": self.neq, "F": self.neq, "Kdiag": self.neq,
             "heat_F": self.hneq}.get(name, self.nno)
        out = np.zeros(n)
        lib().orc_get(self._o, GET[name], _p(out))
        return out

    def kmul(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.neq)
        lib().orc_kmul(self._o, _p(x), _p(y))
        return y

    def gmul(self, p):
        p = np.ascontiguousarray(p, np.float64)
        y = np.zeros(self.neq)
        lib().orc_gmul(self._o, _p(p), _p(y))
        return y

    def gtmul(self, x):
        x = np.ascontiguousarray(x, np.float64)
        p = np.zeros(self.nel)
        lib().orc_gtmul(self._o, _p(x), _p(p))
        return p

    def cg_sample(self, n):
        return lib().orc_cg_sample(self._o, n)


def run(path, steps=1, threads=1):
    """Run `steps` time steps from the configured initial temperature."""
    o = Oracle(path, threads)
    out = {"stats": []}
    for _ in range(steps):
        out["stats"].append(o.step())
    for k in ("T", "V0", "V1", "P", "d", "stress", "vis"):
        out[k] = o.get(k)
    o.close()
    return out
