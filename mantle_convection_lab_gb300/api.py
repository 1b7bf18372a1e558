"""Python binding of the C ABI in include/mclg.h (ctypes; no torch needed).

The reference drives its hot path as a fixed sequence of argument-less calls
over one global struct (Main.c:55-64).  `Model` exposes the same calls with
the same names over one device-resident context:

    m = Model(Config.from_input("run.input"))
    m.initial_temperature()
    for step in range(cfg.max_timestep + 1):
        m.buoyancy_force(); m.viscosity(); m.velocity_pressure_KGF_matrix()
        st = m.solve_velocity_pressure()
        m.output()                      # every save_spacing steps, Output.c format
        m.update_temperature()

Every call goes to libmclg.so; if the library is missing or no GPU is
visible the call raises -- there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libmclg.so")

OK, CAP_REACHED, NAN, BREAKDOWN, BAD_INPUT, CUDA_ERROR, IO_ERROR, NO_DEVICE = range(8)

FIELDS = {"T": 0, "V0": 1, "V1": 2, "P": 3, "d": 4, "stress": 5, "vis": 6, "buoyancy": 7, "F": 8,
          "Kdiag": 9, "BAB": 10, "tau0": 11, "tau1": 12, "heat_F": 13, "X0": 14, "X1": 15, "gs": 16}
MESH = {"sizes": 0, "Mcode": 1, "node": 2, "ien": 3, "id": 4, "heat_id": 5, "lm": 6, "hang": 7,
        "v_bc": 8, "T_bc": 9, "interp": 10, "project": 11, "gs_wave": 12, "nb": 13, "kslot": 14}
NB_WIDTH = 25   # the width of the "nb" lists
MESH_REAL = {"X": 0, "jacobi": 1, "area": 2, "v_bc_val": 3, "T_bc_val": 4}
OUT_TEXT, OUT_BINARY = 1, 2


class MclgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class Config(C.Structure):
    """mclg_config: the .input keys of Input.c:3-99 plus the GB300 options."""
    _fields_ = [
        ("data_dir", C.c_char * 256), ("solver", C.c_char * 8), ("level", C.c_int), ("mg_min_level", C.c_int),
        ("nprox", C.c_int), ("nproz", C.c_int), ("model_length", C.c_double), ("model_height", C.c_double),
        ("top_v_bc", C.c_char * 2), ("bot_v_bc", C.c_char * 2), ("lef_v_bc", C.c_char * 2),
        ("rig_v_bc", C.c_char * 2), ("top_v_bc_val", C.c_double * 2), ("bot_v_bc_val", C.c_double * 2),
        ("lef_v_bc_val", C.c_double * 2), ("rig_v_bc_val", C.c_double * 2), ("top_T_bc", C.c_char),
        ("bot_T_bc", C.c_char), ("lef_T_bc", C.c_char), ("rig_T_bc", C.c_char), ("top_T_bc_val", C.c_double),
        ("bot_T_bc_val", C.c_double), ("lef_T_bc_val", C.c_double), ("rig_T_bc_val", C.c_double),
        ("T_ini", C.c_int), ("T_mantle", C.c_double), ("T_mantle_perturb", C.c_double),
        ("T_wave_number", C.c_int), ("Rayleigh", C.c_double), ("A", C.c_double), ("refT", C.c_double),
        ("lower_mantle_jump", C.c_double), ("max_timestep", C.c_int), ("save_spacing", C.c_int),
        ("Q", C.c_double), ("theta", C.c_double), ("AMR", C.c_int), ("cg_precondition", C.c_int),
        ("accuracy", C.c_double), ("auto_accuracy", C.c_int), ("citcom_solver_accu", C.c_double),
        ("develop_mode", C.c_int), ("check_v_only", C.c_int), ("max_citcom_cycle", C.c_int),
        ("max_cg_cycle", C.c_int), ("zero_P", C.c_int), ("lg_mul", C.c_int), ("grain_damage", C.c_int),
        ("old_T_file", C.c_char * 1024), ("old_T_timestep", C.c_int), ("ic_kind", C.c_int),
        ("ic_seed", C.c_uint64), ("ic_noise", C.c_double), ("ic_bl_thickness", C.c_double),
        ("ic_mode_amp", C.c_double), ("ic_modes", C.c_int), ("precision", C.c_int),
        ("stokes_rtol", C.c_double), ("warm_start", C.c_int), ("vis_min", C.c_double),
        ("vis_max", C.c_double), ("mg_smooth", C.c_int), ("mg_omega", C.c_double),
        ("mg_coarse", C.c_int), ("outer_rtol", C.c_double), ("inner_rtol", C.c_double),
        ("max_refine", C.c_int), ("max_outer", C.c_int), ("max_inner", C.c_int),
        ("mg_eta_avg", C.c_int), ("mg_block_n", C.c_int), ("guess_smooth", C.c_int),
        ("stokes_method", C.c_int), ("mg_cycle", C.c_int), ("mg_finest_iteration", C.c_int),
        ("mg_coarse_iteration", C.c_int), ("lowest_vis", C.c_double), ("highest_vis", C.c_double),
        ("mg_smooth_coarse", C.c_int), ("mg_smoother", C.c_int), ("mg_cheb_lmax", C.c_double),
        ("mg_cheb_ratio", C.c_double), ("mg_fine_levels", C.c_int),
    ]

    @classmethod
    def defaults(cls):
        c = cls()
        lib().mclg_config_defaults(C.byref(c))
        return c

    @classmethod
    def from_input(cls, path):
        """setup_parser + read_input_file (Parsing.c:54-141, Input.c:3-99)."""
        c = cls()
        _check(lib().mclg_config_from_input(os.fsencode(path), C.byref(c)), "config_from_input")
        return c


class StepStats(C.Structure):
    _fields_ = [
        ("timestep", C.c_int), ("uzawa_cycles", C.c_int), ("cg_cycles", C.c_int), ("heat_cg_cycles", C.c_int),
        ("status", C.c_int), ("dv", C.c_double), ("dp", C.c_double), ("dt", C.c_double),
        ("model_time", C.c_double), ("res_momentum", C.c_double), ("res_continuity", C.c_double),
        ("ms_stokes", C.c_double), ("ms_heat", C.c_double), ("ms_total", C.c_double),
        ("kernel_launches", C.c_longlong), ("solver_kernel_ms", C.c_double),
        ("solver_kernel_launches", C.c_longlong), ("refine_passes", C.c_int),
        ("guess_used", C.c_int), ("res_guess_learned", C.c_double), ("res_guess_prev", C.c_double),
        ("ms_guess", C.c_double), ("warm_alpha", C.c_double), ("warm_beta", C.c_double),
        ("remesh_ms_numbering", C.c_double), ("remesh_ms_lists", C.c_double), ("remesh_ms_state", C.c_double),
        ("remesh_ms_wait", C.c_double), ("remesh_ms_carry", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_LIB = None


def lib():
    """Load libmclg.so (built in-tree by __graft_entry__.build()); raise if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise MclgError(BAD_INPUT, f"{LIB_PATH} is missing: run __graft_entry__.build() first")
    L = C.CDLL(LIB_PATH)
    vp, ip, dp, sz = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_size_t
    fp = C.POINTER(C.c_float)
    sig = {
        "mclg_config_defaults": (None, [vp]), "mclg_config_from_input": (C.c_int, [C.c_char_p, vp]),
        "mclg_config_sizeof": (sz, []), "mclg_step_stats_sizeof": (sz, []),
        "mclg_create": (C.c_int, [C.POINTER(vp), vp]), "mclg_destroy": (None, [vp]),
        "mclg_status_string": (C.c_char_p, [C.c_int]), "mclg_last_error": (C.c_char_p, []),
        "mclg_initial_temperature": (C.c_int, [vp]), "mclg_buoyancy_force": (C.c_int, [vp]),
        "mclg_viscosity": (C.c_int, [vp]), "mclg_velocity_pressure_KGF_matrix": (C.c_int, [vp]),
        "mclg_solve_velocity_pressure": (C.c_int, [vp, vp]), "mclg_update_temperature": (C.c_int, [vp, vp]),
        "mclg_solve_velocity_pressure_noalloc": (C.c_int, [vp, vp]),
        "mclg_output": (C.c_int, [vp, C.c_char_p, C.c_int]), "mclg_step": (C.c_int, [vp, C.c_int, vp]),
        "mclg_step_host": (C.c_int, [vp, dp, dp, dp, dp, vp]),
        "mclg_get_field": (C.c_int, [vp, C.c_int, C.c_int, dp, sz]),
        "mclg_set_field": (C.c_int, [vp, C.c_int, C.c_int, dp, sz]),
        "mclg_get_mesh": (C.c_int, [vp, C.c_int, C.c_int, ip, sz]),
        "mclg_mesh_new": (C.c_int, [C.POINTER(vp), vp]), "mclg_mesh_delete": (None, [vp]),
        "mclg_mesh_get": (C.c_int, [vp, C.c_int, C.c_int, ip, sz]),
        "mclg_mesh_get_real": (C.c_int, [vp, C.c_int, C.c_int, dp, sz]),
        "mclg_mesh_initial_temperature": (C.c_int, [vp, C.c_int, dp, sz]),
        "mclg_mesh_write_output": (C.c_int, [vp, C.c_char_p, C.c_int, dp, dp, dp, dp, dp, sz]),
        "mclg_stokes_matvec": (C.c_int, [vp, C.c_int, dp, dp]), "mclg_stokes_G": (C.c_int, [vp, C.c_int, dp, dp]),
        "mclg_stokes_GT": (C.c_int, [vp, C.c_int, dp, dp]), "mclg_heat_matvec": (C.c_int, [vp, C.c_int, dp, dp]),
        "mclg_cnn_create": (C.c_int, [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong]),
        "mclg_cnn_destroy": (None, [vp]), "mclg_cnn_num_params": (sz, [vp]),
        "mclg_cnn_shape": (C.c_int, [vp, ip, ip, ip, ip]),
        "mclg_cnn_get_params": (C.c_int, [vp, fp, sz]), "mclg_cnn_set_params": (C.c_int, [vp, fp, sz]),
        "mclg_cnn_forward": (C.c_int, [vp, fp, C.c_int, C.c_int, C.c_int, fp]),
        "mclg_cnn_gradient": (C.c_int, [vp, fp, fp, C.c_int, C.c_int, C.c_int, dp, fp, sz]),
        "mclg_cnn_adam_step": (C.c_int, [vp, fp, sz, C.c_float]),
        "mclg_cnn_train": (C.c_int, [vp, fp, fp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                     C.c_ulonglong, fp]),
        "mclg_cnn_save": (C.c_int, [vp, C.c_char_p]), "mclg_cnn_load": (C.c_int, [C.POINTER(vp), C.c_char_p]),
        "mclg_checkpoint_save": (C.c_int, [vp, C.c_char_p]), "mclg_checkpoint_load": (C.c_int, [vp, C.c_char_p]),
        "mclg_restart": (C.c_int, [C.POINTER(vp), vp, C.c_char_p]), "mclg_get_time": (C.c_int, [vp, ip, dp]),
        "mclg_output_async": (C.c_int, [vp, C.c_char_p, C.c_int, C.c_int]), "mclg_output_wait": (C.c_int, [vp]),
        "mclg_guess_set": (C.c_int, [vp, C.c_int, C.c_int, vp]),
        "mclg_create_leaves": (C.c_int, [C.POINTER(vp), vp, ip, sz]),
        "mclg_amr_flags": (C.c_int, [vp, C.c_double, C.POINTER(C.c_ubyte), sz, dp]),
        "mclg_amr_remesh": (C.c_int, [vp, C.c_double, C.c_int, C.c_int, C.POINTER(sz)]),
        "mclg_amr_remesh_begin": (C.c_int, [vp, C.c_double, C.c_int, C.c_int]),
        "mclg_amr_remesh_end": (C.c_int, [vp, C.POINTER(sz)]),
        "mclg_mesh_new_leaves": (C.c_int, [C.POINTER(vp), vp, ip, sz]),
        "mclg_mesh_new_leaves_device": (C.c_int, [C.POINTER(vp), vp, ip, sz]),
        "mclg_mesh_diff": (C.c_int, [vp, vp, C.c_char_p, sz]),
        "mclg_mesh_amr_leaves": (C.c_int, [vp, C.POINTER(C.c_ubyte), sz, C.c_int, C.c_int, ip, sz, C.POINTER(sz)]),
        "mclg_amr_leaves": (C.c_int, [vp, C.POINTER(C.c_ubyte), sz, C.c_int, C.c_int, ip, sz, C.POINTER(sz)]),
        "mclg_mesh_transfer": (C.c_int, [vp, dp, sz, vp, dp, sz]),
        "mclg_mesh_transfer_elem": (C.c_int, [vp, dp, sz, vp, dp, sz]),
        "mclg_mesh_qt_get": (C.c_int, [vp, C.c_int, C.c_int, vp, sz]),
        "mclg_grain_new": (C.c_int, [C.POINTER(vp)]),
        "mclg_grain_update": (C.c_int, [vp, C.c_int, dp, dp, dp, dp, C.c_double, C.c_double, C.c_double,
                                        C.c_double, C.c_int]),
        "mclg_grain_get": (C.c_int, [vp, dp, sz]),
        "mclg_grain_delete": (None, [vp]),
        "mclg_ensemble_create": (C.c_int, [C.POINTER(vp), vp, C.c_int]), "mclg_ensemble_destroy": (None, [vp]),
        "mclg_ensemble_create_amr": (C.c_int, [C.POINTER(vp), vp, ip, C.c_int]),
        "mclg_ensemble_graph": (C.c_int, [vp]),
        "mclg_ensemble_size": (C.c_int, [vp]), "mclg_ensemble_member": (C.c_int, [vp, C.c_int, C.POINTER(vp)]),
        "mclg_ensemble_initial_temperature": (C.c_int, [vp]),
        "mclg_ensemble_step": (C.c_int, [vp, vp, ip]),
        "mclg_guess_sample": (C.c_int, [vp, fp, sz, fp, sz]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if L.mclg_config_sizeof() != C.sizeof(Config) or L.mclg_step_stats_sizeof() != C.sizeof(StepStats):
        raise MclgError(BAD_INPUT, "ctypes layout of mclg_config/mclg_step_stats does not match libmclg.so")
    _LIB = L
    return L


def _check(rc, what):
    if rc not in (OK, CAP_REACHED):
        L = lib()
        raise MclgError(rc, f"{what}: {L.mclg_status_string(rc).decode()}: {L.mclg_last_error().decode()}")
    return rc


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


GUESS_OFF, GUESS_RECORD, GUESS_LEARNED, GUESS_FORCED = 0, 1, 2, 3
GUESS_CIN, GUESS_COUT = 8, 3


class Cnn:
    """The learned-guess network (mclg_cnn_*): 3x3 convolutions, BF16 weights,
    FP32 accumulation, trained on the device by the library's own kernels."""

    def __init__(self, cin=GUESS_CIN, width=32, depth=6, cout=GUESS_COUT, seed=0, _handle=None):
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
        else:
            _check(lib().mclg_cnn_create(C.byref(self._h), cin, width, depth, cout, seed), "cnn_create")
        a = [C.c_int() for _ in range(4)]
        _check(lib().mclg_cnn_shape(self._h, *[C.byref(x) for x in a]), "cnn_shape")
        self.cin, self.width, self.depth, self.cout = (x.value for x in a)
        self.nparam = int(lib().mclg_cnn_num_params(self._h))

    @classmethod
    def load(cls, path):
        h = C.c_void_p()
        _check(lib().mclg_cnn_load(C.byref(h), os.fsencode(path)), "cnn_load")
        return cls(_handle=h)

    def save(self, path):
        _check(lib().mclg_cnn_save(self._h, os.fsencode(path)), "cnn_save")

    def close(self):
        if self._h:
            lib().mclg_cnn_destroy(self._h)
            self._h = C.c_void_p()

    __del__ = close

    def params(self):
        out = np.zeros(self.nparam, np.float32)
        _check(lib().mclg_cnn_get_params(self._h, _fptr(out), out.size), "cnn_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        _check(lib().mclg_cnn_set_params(self._h, _fptr(p), p.size), "cnn_set_params")

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        b, c, h, w = x.shape
        y = np.zeros((b, self.cout, h, w), np.float32)
        _check(lib().mclg_cnn_forward(self._h, _fptr(x), b, h, w, _fptr(y)), "cnn_forward")
        return y

    def gradient(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        b, c, h, w = x.shape
        g = np.zeros(self.nparam, np.float32)
        loss = C.c_double()
        _check(lib().mclg_cnn_gradient(self._h, _fptr(x), _fptr(t), b, h, w, C.byref(loss), _fptr(g), g.size),
               "cnn_gradient")
        return loss.value, g

    def adam_step(self, g, lr):
        g = np.ascontiguousarray(g, np.float32)
        _check(lib().mclg_cnn_adam_step(self._h, _fptr(g), g.size, lr), "cnn_adam_step")

    def train(self, x, t, batch=16, iters=100, lr=1e-3, seed=0):
        """Adam on the mean squared error; returns the loss of every iteration."""
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        n, c, h, w = x.shape
        trace = np.zeros(max(iters, 1), np.float32)
        _check(lib().mclg_cnn_train(self._h, _fptr(x), _fptr(t), n, h, w, batch, iters, lr, seed, _fptr(trace)),
               "cnn_train")
        return trace[:iters]


def _uptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_ubyte))


class GrainSize:
    """Grain-size rheology (grain_damage=1) on the host: the reference's routine
    with its first-call flag, clock and nodal grain size (mclg_grain_*)."""

    def __init__(self):
        self._g = C.c_void_p()
        _check(lib().mclg_grain_new(C.byref(self._g)), "grain_new")
        self.nno = None

    def update(self, X, T, stress, vis, model_time, Ra, lowest_vis, highest_vis, threads=4):
        """One call of the routine; returns the (stress, vis) it leaves."""
        X = np.ascontiguousarray(X, np.float64)
        T = np.ascontiguousarray(T, np.float64)
        stress = np.array(stress, np.float64)
        vis = np.array(vis, np.float64)
        self.nno = T.size
        _check(lib().mclg_grain_update(self._g, T.size, _dptr(X), _dptr(T), _dptr(stress), _dptr(vis), model_time,
                                       Ra, lowest_vis, highest_vis, threads), "grain_update")
        return stress, vis

    def grain_size(self):
        out = np.zeros(self.nno)
        _check(lib().mclg_grain_get(self._g, _dptr(out), out.size), "grain_get")
        return out

    def close(self):
        if self._g:
            lib().mclg_grain_delete(self._g)
            self._g = C.c_void_p()

    def __del__(self):
        self.close()


class Mesh:
    """Host-only mesh of Main.c:33-52 (quadtree, numbering, BC codes, hanging nodes).
    leaves: build from finest-level Morton start codes instead of develop_mode;
    device=True numbers that leaf set on the current CUDA device instead (the
    same arrays, byte for byte)."""

    def __init__(self, config, leaves=None, device=False):
        self._h = C.c_void_p()
        self.config = config
        if leaves is None:
            if device:
                raise MclgError(BAD_INPUT, "the device numbering takes a leaf list")
            _check(lib().mclg_mesh_new(C.byref(self._h), C.byref(config)), "mesh_new")
        else:
            lv = np.ascontiguousarray(leaves, np.int32)
            fn = lib().mclg_mesh_new_leaves_device if device else lib().mclg_mesh_new_leaves
            _check(fn(C.byref(self._h), C.byref(config), _iptr(lv), lv.size), "mesh_new_leaves")
        s = self.get("sizes")
        self.nel, self.nno, self.neq, self.heat_neq, self.nh, self.gnox, self.gnoz, self.max_level = map(int, s)

    def close(self):
        if self._h:
            lib().mclg_mesh_delete(self._h)
            self._h = C.c_void_p()

    __del__ = close

    def _size(self, which, lev):
        if which == "sizes":
            return 8
        s = np.zeros(8, np.int32)
        _check(lib().mclg_mesh_get(self._h, 0, lev, _iptr(s), 8), "mesh_get")
        nel, nno, neq, hneq, nh = (int(v) for v in s[:5])
        return {"Mcode": nel, "node": nno, "ien": 4 * nel, "id": 2 * nno, "heat_id": nno, "lm": 8 * nel,
                "hang": 3 * nh, "v_bc": 2 * nno, "T_bc": nno, "X": 2 * nno, "jacobi": nel, "area": nel,
                "v_bc_val": 2 * nno, "T_bc_val": nno, "interp": 5 * neq, "project": neq, "gs_wave": nno,
                "nb": NB_WIDTH * nno, "kslot": 16 * nel}[which]

    def get(self, which, lev=-1):
        n = self._size(which, lev)
        if which in MESH_REAL:
            out = np.zeros(n, np.float64)
            _check(lib().mclg_mesh_get_real(self._h, MESH_REAL[which], lev, _dptr(out), n), "mesh_get_real")
            return out
        out = np.zeros(n, np.int32)
        _check(lib().mclg_mesh_get(self._h, MESH[which], lev, _iptr(out), n), "mesh_get")
        return out

    def diff(self, other):
        """None when every array of every level equals other's byte for byte,
        else the name of the first one that differs."""
        buf = C.create_string_buffer(128)
        return buf.value.decode() if lib().mclg_mesh_diff(self._h, other._h, buf, 128) else None

    def initial_temperature(self, lev=-1):
        n = self._size("node", lev)
        out = np.zeros(n, np.float64)
        _check(lib().mclg_mesh_initial_temperature(self._h, lev, _dptr(out), n), "mesh_initial_temperature")
        return out

    def amr_leaves(self, flags, base_level, target_level):
        """Leaves of the refined tree for per-element flags of the finest level."""
        f = np.ascontiguousarray(flags, np.uint8)
        cap = 1 << (2 * (self.max_level - 1))
        out = np.zeros(cap, np.int32)
        n = C.c_size_t()
        _check(lib().mclg_mesh_amr_leaves(self._h, _uptr(f), f.size, base_level, target_level, _iptr(out), cap,
                                           C.byref(n)), "mesh_amr_leaves")
        return out[:n.value].copy()

    def transfer(self, T, to):
        """T (finest-level nodes of this mesh) interpolated onto `to`'s nodes."""
        T = np.ascontiguousarray(T, np.float64)
        out = np.zeros(to.nno)
        _check(lib().mclg_mesh_transfer(self._h, _dptr(T), T.size, to._h, _dptr(out), out.size), "mesh_transfer")
        return out

    def qt(self, lev=-1):
        """The refined-mesh solver's host lists of one level (mclg_mesh_qt_get):
        kind, and the contribution lists that assemble C^T K C."""
        def fetch(which, n, dtype):
            out = np.zeros(n, dtype)
            _check(lib().mclg_mesh_qt_get(self._h, lev, which, out.ctypes.data_as(C.c_void_p), n), "mesh_qt_get")
            return out
        nno, width, n_rc, n_ex = (int(v) for v in fetch(0, 4, np.int32))
        return {"nno": nno, "width": width, "kind": fetch(1, 2 * nno, np.int32),
                "rc_off": fetch(2, nno + 1, np.int32), "rc_tgt": fetch(3, n_rc, np.int32),
                "rc_src": fetch(4, n_rc, np.int32), "rc_w": fetch(5, n_rc, np.float64),
                "rnb": fetch(6, width * nno, np.int32), "rcnt": fetch(7, nno, np.int32)}

    def transfer_elem(self, P, to):
        """An element field of this mesh (the pressure) onto `to`'s elements: the
        area mean of P over each new element."""
        P = np.ascontiguousarray(P, np.float64)
        out = np.zeros(to.nel)
        _check(lib().mclg_mesh_transfer_elem(self._h, _dptr(P), P.size, to._h, _dptr(out), out.size),
               "mesh_transfer_elem")
        return out

    def write_output(self, data_dir, timestep, T, V0, V1, stress, vis):
        """Output.c's text files for host fields of the finest level (G.node order)."""
        f = [np.ascontiguousarray(a, np.float64) for a in (T, V0, V1, stress, vis)]
        n = f[0].size
        if any(a.size != n for a in f):
            raise MclgError(BAD_INPUT, "write_output: fields differ in length")
        _check(lib().mclg_mesh_write_output(self._h, data_dir.encode(), int(timestep), *map(_dptr, f), n),
               "mesh_write_output")


class Model:
    """One device-resident model; method names follow the reference's calls."""

    def __init__(self, config, _handle=None, leaves=None, restart=None):
        """restart: a checkpoint file (mclg_restart): the model is built on its mesh and takes its state."""
        self.config = config
        self._c = C.c_void_p()
        self._owned = _handle is None
        if _handle is not None:
            self._c = _handle
        elif restart is not None:
            _check(lib().mclg_restart(C.byref(self._c), C.byref(config), os.fsencode(restart)), "restart")
        elif leaves is not None:
            lv = np.ascontiguousarray(leaves, np.int32)
            _check(lib().mclg_create_leaves(C.byref(self._c), C.byref(config), _iptr(lv), lv.size), "create_leaves")
        else:
            _check(lib().mclg_create(C.byref(self._c), C.byref(config)), "create")
        s = self.mesh("sizes")
        self.nel, self.nno, self.neq, self.heat_neq, self.nh, self.gnox, self.gnoz, self.max_level = map(int, s)
        self.timestep = 0
        if restart is not None:
            self.timestep = self._timestep()

    def _timestep(self):
        return self.time()[0]

    def time(self):
        """(G.timestep, G.model_time) of the model."""
        ts, mt = C.c_int(), C.c_double()
        _check(lib().mclg_get_time(self._c, C.byref(ts), C.byref(mt)), "get_time")
        return ts.value, mt.value

    def checkpoint(self, path):
        """Write the whole state to `path` (mclg_checkpoint_save)."""
        _check(lib().mclg_checkpoint_save(self._c, os.fsencode(path)), "checkpoint_save")

    def load_checkpoint(self, path):
        """Take the state of a checkpoint written on the same mesh (mclg_checkpoint_load)."""
        _check(lib().mclg_checkpoint_load(self._c, os.fsencode(path)), "checkpoint_load")
        self.timestep = self._timestep()

    def close(self):
        if self._c and self._owned:
            lib().mclg_destroy(self._c)
        self._c = C.c_void_p()

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # --- the Main.c:55-64 sequence ---
    def initial_temperature(self):
        _check(lib().mclg_initial_temperature(self._c), "initial_temperature")
        self.timestep = 0

    def buoyancy_force(self):
        _check(lib().mclg_buoyancy_force(self._c), "buoyancy_force")

    def viscosity(self):
        _check(lib().mclg_viscosity(self._c), "viscosity")

    def velocity_pressure_KGF_matrix(self):
        _check(lib().mclg_velocity_pressure_KGF_matrix(self._c), "velocity_pressure_KGF_matrix")

    def solve_velocity_pressure(self):
        st = StepStats()
        _check(lib().mclg_solve_velocity_pressure(self._c, C.byref(st)), "solve_velocity_pressure")
        return st

    def solve_velocity_pressure_noalloc(self):
        """The same solve with library-resident scratch: allocates no device memory."""
        st = StepStats()
        _check(lib().mclg_solve_velocity_pressure_noalloc(self._c, C.byref(st)),
               "solve_velocity_pressure_noalloc")
        return st

    def update_temperature(self):
        st = StepStats()
        _check(lib().mclg_update_temperature(self._c, C.byref(st)), "update_temperature")
        self.timestep += 1
        return st

    def output(self, data_dir=None, timestep=None):
        d = None if data_dir is None else os.fsencode(data_dir)
        _check(lib().mclg_output(self._c, d, self.timestep if timestep is None else timestep), "output")

    def output_async(self, data_dir=None, timestep=None, text=True, binary=False):
        """output() off the critical path (mclg_output_async); output_wait() for completion."""
        d = None if data_dir is None else os.fsencode(data_dir)
        flags = (OUT_TEXT if text else 0) | (OUT_BINARY if binary else 0)
        _check(lib().mclg_output_async(self._c, d, self.timestep if timestep is None else timestep, flags),
               "output_async")

    def output_wait(self):
        _check(lib().mclg_output_wait(self._c), "output_wait")

    def step(self, write_output=False):
        st = StepStats()
        _check(lib().mclg_step(self._c, int(bool(write_output)), C.byref(st)), "step")
        self.timestep += 1
        return st

    def step_host(self, T_in, T_out, V_out, P_out):
        st = StepStats()
        _check(lib().mclg_step_host(self._c, _dptr(T_in), _dptr(T_out), _dptr(V_out), _dptr(P_out),
                                    C.byref(st)), "step_host")
        self.timestep += 1
        return st

    # --- state ---
    def _fsize(self, which):
        return {"T": self.nno, "V0": self.nno, "V1": self.nno, "P": self.nel, "d": self.neq,
                "stress": self.nno, "vis": self.nno, "buoyancy": self.nno, "F": self.neq, "Kdiag": self.neq,
                "BAB": self.nel, "tau0": self.nel, "tau1": self.nel, "heat_F": self.heat_neq,
                "X0": self.nno, "X1": self.nno, "gs": self.nno}[which]

    def get(self, which, lev=-1):
        """A field of the finest level; with solver="mg", T and vis of a coarser level `lev` too."""
        n = self._fsize(which) if lev < 0 or lev == self.max_level - 1 else self.mesh("sizes", lev)[1]
        out = np.zeros(n, np.float64)
        _check(lib().mclg_get_field(self._c, FIELDS[which], lev, _dptr(out), out.size), f"get {which}")
        return out

    def set(self, which, values):
        a = np.ascontiguousarray(values, np.float64)
        _check(lib().mclg_set_field(self._c, FIELDS[which], -1, _dptr(a), a.size), f"set {which}")

    def mesh(self, which, lev=-1):
        if which == "sizes":
            n = 8
        else:
            n = {"Mcode": self.nel, "node": self.nno, "ien": 4 * self.nel, "id": 2 * self.nno,
                 "heat_id": self.nno, "lm": 8 * self.nel, "hang": 3 * self.nh, "v_bc": 2 * self.nno,
                 "T_bc": self.nno}[which]
        out = np.zeros(n, np.int32)
        _check(lib().mclg_get_mesh(self._c, MESH[which], lev, _iptr(out), n), f"mesh {which}")
        return out

    # --- single operators ---
    def stokes_matvec(self, x, lev=-1):
        """K x on the finest level; with solver="mg" on a coarser level `lev` too."""
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.neq if lev < 0 or lev == self.max_level - 1 else self.mesh("sizes", lev)[2])
        _check(lib().mclg_stokes_matvec(self._c, lev, _dptr(x), _dptr(y)), "stokes_matvec")
        return y

    def stokes_G(self, p):
        p = np.ascontiguousarray(p, np.float64)
        y = np.zeros(self.neq)
        _check(lib().mclg_stokes_G(self._c, -1, _dptr(p), _dptr(y)), "stokes_G")
        return y

    def stokes_GT(self, x):
        x = np.ascontiguousarray(x, np.float64)
        p = np.zeros(self.nel)
        _check(lib().mclg_stokes_GT(self._c, -1, _dptr(x), _dptr(p)), "stokes_GT")
        return p

    def amr_flags(self, frac=0.2):
        """Per finest-level element: |grad T| > frac * max (device); returns (flags, max)."""
        f = np.zeros(self.nel, np.uint8)
        gmax = C.c_double()
        _check(lib().mclg_amr_flags(self._c, frac, _uptr(f), f.size, C.byref(gmax)), "amr_flags")
        return f, gmax.value

    def amr_leaves(self, flags, base_level, target_level):
        """Leaves of the refined tree for per-element flags of the finest level,
        built on the device (Mesh.amr_leaves builds the same on the host)."""
        f = np.ascontiguousarray(flags, np.uint8)
        cap = 1 << (2 * (self.max_level - 1))
        out = np.zeros(cap, np.int32)
        n = C.c_size_t()
        _check(lib().mclg_amr_leaves(self._c, _uptr(f), f.size, base_level, target_level, _iptr(out), cap,
                                     C.byref(n)), "amr_leaves")
        return out[:n.value].copy()

    def remesh(self, frac, base_level, target_level):
        """Refine by |grad T| and rebuild the model on the new mesh in place."""
        n = C.c_size_t()
        _check(lib().mclg_amr_remesh(self._c, frac, base_level, target_level, C.byref(n)), "amr_remesh")
        s = self.mesh("sizes")
        self.nel, self.nno, self.neq, self.heat_neq, self.nh, self.gnox, self.gnoz, self.max_level = map(int, s)
        return n.value

    def remesh_begin(self, frac, base_level, target_level):
        """First half of remesh(): flags and leaves now, the new mesh built on a host thread."""
        _check(lib().mclg_amr_remesh_begin(self._c, frac, base_level, target_level), "amr_remesh_begin")

    def remesh_end(self):
        """Second half: wait for the new mesh, carry the current fields over, swap it in."""
        n = C.c_size_t()
        _check(lib().mclg_amr_remesh_end(self._c, C.byref(n)), "amr_remesh_end")
        s = self.mesh("sizes")
        self.nel, self.nno, self.neq, self.heat_neq, self.nh, self.gnox, self.gnoz, self.max_level = map(int, s)
        return n.value

    def guess_set(self, mode, grid=128, net=None):
        """Learned initial guess: GUESS_OFF, GUESS_RECORD (features and targets
        only) or GUESS_LEARNED (needs `net`)."""
        self._guess_net = net   # keep the network alive while the context uses it
        self._guess_grid = grid
        _check(lib().mclg_guess_set(self._c, mode, grid, net._h if net is not None else None), "guess_set")

    def guess_sample(self):
        """(features [8, g+1, g+1], target [3, g+1, g+1]) of the last solve."""
        n = self._guess_grid + 1
        x = np.zeros((GUESS_CIN, n, n), np.float32)
        y = np.zeros((GUESS_COUT, n, n), np.float32)
        _check(lib().mclg_guess_sample(self._c, _fptr(x), x.size, _fptr(y), y.size), "guess_sample")
        return x, y

    def heat_matvec(self, which, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.heat_neq)
        _check(lib().mclg_heat_matvec(self._c, {"K": 0, "C": 1}[which], _dptr(x), _dptr(y)), "heat_matvec")
        return y


class Ensemble:
    """Independent models stepped together: one batched solver launch per step
    (mclg_ensemble_*) for the members on uniform meshes; amr_levels[i] > 0 refines
    member i from its configuration's grid by |grad T| (mclg_ensemble_create_amr)."""

    def __init__(self, configs, amr_levels=None):
        arr = (Config * len(configs))(*configs)
        self._e = C.c_void_p()
        if amr_levels is None:
            _check(lib().mclg_ensemble_create(C.byref(self._e), arr, len(configs)), "ensemble_create")
        else:
            lv = np.ascontiguousarray(amr_levels, np.int32)
            if lv.size != len(configs):
                raise MclgError(BAD_INPUT, "amr_levels: one entry per member")
            _check(lib().mclg_ensemble_create_amr(C.byref(self._e), arr, _iptr(lv), len(configs)),
                   "ensemble_create_amr")
        self.n = len(configs)
        self.members = []
        for i in range(self.n):
            h = C.c_void_p()
            _check(lib().mclg_ensemble_member(self._e, i, C.byref(h)), "ensemble_member")
            self.members.append(Model(configs[i], _handle=h))
        self.cluster_used = 0

    def close(self):
        if self._e:
            for m in self.members:
                m.close()
            lib().mclg_ensemble_destroy(self._e)
            self._e = C.c_void_p()

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def initial_temperature(self):
        _check(lib().mclg_ensemble_initial_temperature(self._e), "ensemble_initial_temperature")
        for m in self.members:
            m.timestep = 0

    @property
    def graph(self):
        """True when steps replay the captured CUDA graph of the whole step."""
        return bool(lib().mclg_ensemble_graph(self._e))

    def step(self):
        stats = (StepStats * self.n)()
        g = C.c_int()
        _check(lib().mclg_ensemble_step(self._e, stats, C.byref(g)), "ensemble_step")
        self.cluster_used = g.value
        for m in self.members:
            m.timestep += 1
        return list(stats)
