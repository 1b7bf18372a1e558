"""Standalone input and uniform-mesh arrays for the CPU oracle -- test infrastructure.

The oracle (oracle.c via oracle_port.py) normally takes its mesh arrays from
the engine's host mesh builder.  This module gives it the same arrays for
uniform meshes (develop_mode=0, one rank) without loading the engine's
library, so that the CPU baseline of bench.py runs the reference's algorithm
with nothing of the product underneath:

  read_input(path)   the .input keys the oracle needs, read with the getpar
                     dialect (Parsing.c:83-125: '#' comments, name=value pairs,
                     quoted values, the last occurrence of a key wins,
                     Parsing.c:231-243) and the defaults of Input.c:3-99
  UniformMesh(cfg)   the finest level of a uniform mesh:
                     - leaves in Morton order with the level in the low 4 bits
                       (morton / build_quad_tree, Tree.c:67-99, 447-456)
                     - node ids iz + ix*gnoz, all present and sorted
                       (construct_ien, node_index_from_ien,
                       Construct_ien_id_lm.c:3-78)
                     - ien corners (ex,ez) (ex,ez+1) (ex+1,ez+1) (ex+1,ez)
                     - positions ix*dx, iz*dz (node_position, Mesh.c:432-452)
                     - BC codes and values (temperature_bc / velocity_bc,
                       Boundary_condition.c:10-110)
                     - no hanging nodes
  UniformMesh.initial_temperature()  T_ini 0, 1 and the seeded -2 through
                     liboracle.so (the C of Initial_condition.c:3-75 and of the
                     engine's seeded-field header), then the Dirichlet values
                     (apply_T_bc_values, Initial_condition.c:122-136)

tests/test_oracle_standalone.py pins every array against the reference's
dumps and against the engine's builder.
"""
import ctypes as C
import re

import numpy as np

_NUM_INT = re.compile(r"\s*[+-]?\d+")
_NUM_FLT = re.compile(r"\s*[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?|inf|nan)", re.I)


def _tokens(path):
    """setup_parser (Parsing.c:83-125): the (name, value) pairs of a file in order."""
    out = []
    with open(path) as fh:
        for line in fh:
            i, n = 0, len(line)
            while True:
                while i < n and line[i] in " \t":
                    i += 1
                if i >= n or line[i] in "\n#":
                    break
                j = i
                while j < n and line[j] not in "= \n\t":
                    j += 1
                name = line[i:j]
                i = j + 1 if j < n and line[j] == "=" else j
                if i < n and line[i] in "\"'":
                    stops = (line[i],)
                    i += 1
                else:
                    stops = (" ", "\t")
                j = i
                while j < n and line[j] not in stops and line[j] != "\n":
                    j += 1
                out.append((name, line[i:j]))
                i = j + 1 if j < n and line[j] in "\"'" else j
    return out


class InputConfig:
    """The .input keys the oracle reads (Input.c:3-99 defaults), as attributes
    with the engine's Config names; `solver` is bytes, as there."""
    INTS = {"level": 1, "mg_min_level": 1, "nprox": 2, "nproz": 2, "T_ini": 1, "T_wave_number": 6,
            "max_timestep": 0, "AMR": 0, "cg_precondition": 0, "auto_accuracy": 0, "develop_mode": 1,
            "check_v_only": 0, "max_citcom_cycle": 375, "max_cg_cycle": 200, "lg_mul": 0, "grain_damage": 0,
            "zero_P": 1, "ic_kind": 1, "ic_modes": 8, "mg_cycle": 2, "mg_finest_iteration": 4,
            "mg_coarse_iteration": 4}
    FLOATS = {"model_length": 2.0, "model_height": 1.0, "top_T_bc_val": 0.0, "bot_T_bc_val": 1.0,
              "lef_T_bc_val": 0.0, "rig_T_bc_val": 0.0, "T_mantle": 0.5, "T_mantle_perturb": 0.01,
              "Rayleigh": 1e7, "A": 0.0, "refT": 0.5, "lower_mantle_jump": 1.0, "Q": 0.0, "theta": 0.0,
              "accuracy": 0.001, "citcom_solver_accu": 0.001, "ic_noise": 0.0, "ic_bl_thickness": 0.02,
              "ic_mode_amp": 0.005, "vis_min": 0.0, "vis_max": 0.0, "lowest_vis": 1.0, "highest_vis": 1.0}
    VBC = {"top_v_bc": "sv", "bot_v_bc": "sv", "lef_v_bc": "vs", "rig_v_bc": "vs"}
    TBC = {"top_T_bc": "T", "bot_T_bc": "T", "lef_T_bc": "F", "rig_T_bc": "F"}

    def __init__(self, path):
        kv = {}
        for k, v in _tokens(path):
            kv[k] = v                       # the last occurrence wins
        for k, d in self.INTS.items():
            m = _NUM_INT.match(kv[k]) if k in kv else None
            setattr(self, k, int(m.group()) if m else d)
        for k, d in self.FLOATS.items():
            m = _NUM_FLT.match(kv[k]) if k in kv else None
            setattr(self, k, float(m.group()) if m else d)
        for k, d in self.VBC.items():
            s = kv.get(k, d)
            setattr(self, k, (s + "\0\0")[:2].encode() if s else b"\0\0")
            vals = [0.0, 0.0]
            if k + "_val" in kv:            # input_double_vector: missing entries keep 0
                for i, t in enumerate(kv[k + "_val"].split(",")[:2]):
                    m = _NUM_FLT.match(t)
                    if not m:
                        break
                    vals[i] = float(m.group())
            setattr(self, k + "_val", vals)
        for k, d in self.TBC.items():
            s = kv.get(k, d)
            setattr(self, k, s[:1].encode() if s else b"\0")
        self.solver = kv.get("solver", "jc").encode()[:7]
        self.ic_seed = int(_NUM_INT.match(kv["ic_seed"]).group()) if "ic_seed" in kv else 0


def read_input(path):
    return InputConfig(path)


def _spread(v):
    v = v.astype(np.int64) & 0xFFFF
    v = (v | (v << 8)) & 0x00FF00FF
    v = (v | (v << 4)) & 0x0F0F0F0F
    v = (v | (v << 2)) & 0x33333333
    v = (v | (v << 1)) & 0x55555555
    return v


def _compact(v):
    v = v.astype(np.int64) & 0x55555555
    v = (v | (v >> 1)) & 0x33333333
    v = (v | (v >> 2)) & 0x0F0F0F0F
    v = (v | (v >> 4)) & 0x00FF00FF
    v = (v | (v >> 8)) & 0x0000FFFF
    return v


class UniformMesh:
    """Finest level of the uniform mesh of `cfg` (develop_mode=0, one rank).

    With `level` below cfg.level the mesh is the uniform grid of that level
    (2**(level-1) elements per side) and the seeded initial temperature is
    drawn with the node ids of cfg.level's grid, as the engine draws it for a
    coarse uniform base inside a finer tree."""

    def __init__(self, cfg, level=None):
        if cfg.develop_mode != 0 or cfg.nprox * cfg.nproz != 1 or cfg.AMR != 0:
            raise ValueError("UniformMesh covers develop_mode=0 on one rank without AMR")
        self.cfg = cfg
        level = cfg.level if level is None else level
        if not 1 <= level <= cfg.level:
            raise ValueError(f"level {level} outside 1..{cfg.level}")
        self.max_level = level
        self._ic_scale = 1 << (cfg.level - level)
        fl = level - 1
        N = 1 << fl
        self.N = N
        self.gnox = self.gnoz = N + 1
        n = N + 1
        # leaves in Morton order: code k <-> element (ex, ez) with x in the odd bits
        k = np.arange(N * N, dtype=np.int64)
        ex, ez = _compact(k >> 1), _compact(k)
        assert np.array_equal((_spread(ex) << 1) | _spread(ez), k)
        self._arr = {}
        self._arr["Mcode"] = ((k << 4) | fl).astype(np.int32)
        self._arr["node"] = np.arange(n * n, dtype=np.int32)
        ien = np.stack([ez + ex * n, ez + 1 + ex * n, ez + 1 + (ex + 1) * n, ez + (ex + 1) * n])
        self._arr["ien"] = ien.astype(np.int32).ravel()
        gid = np.arange(n * n, dtype=np.int64)
        ix, iz = gid // n, gid % n
        dx = cfg.model_length / float(N)   # G.dx[lev] = length / max_elx[lev] (Mesh.c:419-420)
        dz = cfg.model_height / float(N)
        self._arr["X"] = np.concatenate([ix * dx, iz * dz])
        top, bot = (gid + 1) % n == 0, gid % n == 0
        left, right = gid < n, gid > (n - 1) * n - 1
        tbc = np.full(n * n, ord("N"), np.int32)
        tval = np.zeros(n * n)
        for mask, key in ((top, "top"), (bot & ~top, "bot")):
            tbc[mask] = getattr(cfg, key + "_T_bc")[0]
            tval[mask] = getattr(cfg, key + "_T_bc_val")
        rest = ~top & ~bot
        for mask, key in ((rest & left, "lef"), (rest & ~left & right, "rig")):
            keep = mask & (tbc == ord("T"))
            tbc[mask & ~keep] = getattr(cfg, key + "_T_bc")[0]
            tval[mask] = getattr(cfg, key + "_T_bc_val")
        vbc = np.full((2, n * n), ord("N"), np.int32)
        vval = np.zeros((2, n * n))
        for d in range(2):
            for mask, key in ((top, "top"), (bot & ~top, "bot")):
                vbc[d, mask] = getattr(cfg, key + "_v_bc")[d]
                vval[d, mask] = getattr(cfg, key + "_v_bc_val")[d]
            for mask, key in ((left, "lef"), (~left & right, "rig")):
                keep = mask & (vbc[d] == ord("V"))
                vbc[d, mask & ~keep] = getattr(cfg, key + "_v_bc")[d]
                vval[d, mask] = getattr(cfg, key + "_v_bc_val")[d]
        self._arr["T_bc"] = tbc
        self._arr["T_bc_val"] = tval
        self._arr["v_bc"] = vbc.ravel()
        self._arr["v_bc_val"] = vval.ravel()
        self._arr["hang"] = np.zeros(0, np.int32)

    def get(self, name, lev=None):
        if lev is not None and lev != self.max_level - 1:
            raise ValueError("UniformMesh holds the finest level only")
        return self._arr[name]

    def initial_temperature(self, lev=None):
        from oracle_port import lib
        cfg = self.cfg
        if cfg.T_ini not in (0, 1, -2):
            raise ValueError(f"T_ini={cfg.T_ini}: the standalone oracle input covers 0, 1 and -2")
        X = np.ascontiguousarray(self._arr["X"])
        node = self._arr["node"]
        nn = node.size
        if self._ic_scale > 1:            # the node ids of the finer grid the field is keyed by
            n, k, nf = self.N + 1, self._ic_scale, self.N * self._ic_scale + 1
            node = np.ascontiguousarray(((node % n) * k + (node // n) * k * nf).astype(np.int32))
        T = np.zeros(nn)
        dpar = np.array([cfg.model_length, cfg.model_height, cfg.T_mantle, cfg.T_mantle_perturb, cfg.ic_noise,
                         cfg.ic_bl_thickness, cfg.ic_mode_amp])
        ipar = np.array([cfg.T_wave_number, cfg.ic_kind, cfg.ic_modes], np.int32)
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        lib().orc_initial_temperature(cfg.T_ini, p(dpar), p(ipar), C.c_uint64(cfg.ic_seed), nn, p(X), p(node), p(T))
        fixed = self._arr["T_bc"] == ord("T")
        T[fixed] = self._arr["T_bc_val"][fixed]
        return T
