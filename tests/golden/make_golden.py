"""Generate golden fixtures from the reference built from source.

Runs oracle/_ref/mcc_ref (built by oracle/ref/Makefile from the reference's
own .c files plus the dump harness oracle/ref/harness.c) on small seeded
cases and stores what the harness dumps as compressed .npz fixtures next to
this script, together with the .input file of each case.

    make -C oracle/ref REF=<path to the reference sources>
    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py cfg1_l5    # one case

Keys in <case>.npz:
    mesh/<array>@<lev>       numbering and geometry (harness dump_mesh)
    ops/<array>@<lev>        assembled K, G (CSR), F, Kdiag, BAB, K x, G p, G^T x
    step<k>/<array>          fields after the Stokes solve of step k (with grain_damage=1
                             also gs, the grain size)
    heat<k>/<array>          fields after update_temperature of step k
    series/<name>            per-step scalars: dt, model_time, uzawa cycles, residuals
"""
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from dumpio import read_dump  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "mcc_ref")

BASE = """\
data_dir="./out"
save_spacing=1
nprox=1
nproz=1
model_length=1.0
model_height=1.0
AMR=0
cg_precondition=1
max_citcom_cycle=2000
max_cg_cycle=2000
accuracy=1e-20
citcom_solver_accu=1e-8
solver="cg"
Q=0.0
theta=0.5
top_T_bc=T
top_T_bc_val=0.0
bot_T_bc=T
bot_T_bc_val=1.0
lef_T_bc=F
lef_T_bc_val=0.0
rig_T_bc=F
rig_T_bc_val=0.0
top_v_bc="SV"
top_v_bc_val=0.0,0.0
bot_v_bc="SV"
bot_v_bc_val=0.0,0.0
lef_v_bc="VS"
lef_v_bc_val=0.0,0.0
rig_v_bc="VS"
rig_v_bc_val=0.0,0.0
refT=0.0
T_ini=-2
"""

# name: (extra .input lines, steps to keep in full (None = all), keep coarse levels)
CASES = {
    # configuration 1 (plain method) at 16x16: everything, 4 steps
    "cfg1_l5": ("level=5\nmg_min_level=3\nmax_timestep=3\ndevelop_mode=0\nRayleigh=1e5\nA=0.0\n"
                "ic_kind=1\nic_seed=42\nic_noise=1e-4\nT_mantle_perturb=0.01\nT_wave_number=1\n",
                None, True),
    # configuration 1 at its own size, 64x64, 100 steps
    "cfg1_l7": ("level=7\nmg_min_level=6\nmax_timestep=99\ndevelop_mode=0\nRayleigh=1e5\nA=0.0\n"
                "ic_kind=1\nic_seed=42\nic_noise=1e-4\nT_mantle_perturb=0.01\nT_wave_number=1\n",
                [0, 1, 2, 10, 50, 99], False),
    # boundary-band refinement with hanging nodes and temperature-dependent viscosity
    "hang11_l6": ("level=6\nmg_min_level=4\nmax_timestep=2\ndevelop_mode=11\nRayleigh=1e5\n"
                  "A=0.0\nic_kind=1\nic_seed=7\nic_noise=1e-3\nT_mantle_perturb=0.01\n"
                  "T_wave_number=1\n", None, True),
    # the same mesh with viscosity contrast 1e4; the reference's Uzawa loop runs to its cap
    "hang11v_l6": ("level=6\nmg_min_level=4\nmax_timestep=1\ndevelop_mode=11\nRayleigh=1e6\n"
                   "A=9.210340371976184\nic_kind=1\nic_seed=7\nic_noise=1e-3\nT_mantle_perturb=0.01\n"
                   "T_wave_number=1\nmax_citcom_cycle=60\n", None, False),
    # top-band refinement (2:1 jump across the domain)
    "dev12_l7": ("level=7\nmg_min_level=5\nmax_timestep=0\nmax_citcom_cycle=40\ndevelop_mode=12\nRayleigh=1e5\nA=0.0\n"
                 "ic_kind=1\nic_seed=3\nic_noise=1e-4\nT_mantle_perturb=0.01\nT_wave_number=1\n",
                 None, True),
    # multi-band graded refinement, elements up to 5 levels apart
    "dev13_l8": ("level=8\nmg_min_level=6\nmax_timestep=0\nmax_citcom_cycle=20\ndevelop_mode=13\nRayleigh=1e5\nA=0.0\n"
                 "ic_kind=1\nic_seed=5\nic_noise=1e-4\nT_mantle_perturb=0.01\nT_wave_number=2\n",
                 None, False),
    # lower-half refinement
    "dev14_l7": ("level=7\nmg_min_level=5\nmax_timestep=0\nmax_citcom_cycle=40\ndevelop_mode=14\nRayleigh=1e5\nA=0.0\n"
                 "ic_kind=1\nic_seed=11\nic_noise=1e-4\nT_mantle_perturb=0.01\nT_wave_number=1\n",
                 None, True),
    # the reference's other inner solvers: multigrid V-cycles with Gauss-Seidel smoothing
    # (solver="mg") and plain Gauss-Seidel (solver="gs"), uniform 16x16 and a hanging-node mesh
    "mg_l5": ("level=5\nmg_min_level=2\nmax_timestep=2\ndevelop_mode=0\nRayleigh=1e5\nA=0.0\n"
              "ic_kind=1\nic_seed=42\nic_noise=1e-4\nT_mantle_perturb=0.01\nT_wave_number=1\n"
              "solver=\"mg\"\naccuracy=1e-10\nmax_citcom_cycle=400\n", None, True),
    "gs_l5": ("level=5\nmg_min_level=2\nmax_timestep=1\ndevelop_mode=0\nRayleigh=1e5\nA=0.0\n"
              "ic_kind=1\nic_seed=42\nic_noise=1e-4\nT_mantle_perturb=0.01\nT_wave_number=1\n"
              "solver=\"gs\"\naccuracy=1e-10\nmax_citcom_cycle=400\n", None, True),
    "mg11_l6": ("level=6\nmg_min_level=3\nmax_timestep=0\ndevelop_mode=11\nRayleigh=1e5\nA=0.0\n"
                "ic_kind=1\nic_seed=7\nic_noise=1e-3\nT_mantle_perturb=0.01\nT_wave_number=1\n"
                "solver=\"mg\"\naccuracy=1e-10\nmax_citcom_cycle=400\n", None, True),
    # configuration 3 shape at 32x32: tanh layers + seeded modes, viscosity contrast 1e5
    "vc_l6": ("level=6\nmg_min_level=3\nmax_timestep=2\ndevelop_mode=0\nRayleigh=1e6\n"
              "A=11.512925464970229\nic_kind=2\nic_seed=2024\nic_noise=0.0\nic_bl_thickness=0.02\n"
              "ic_modes=8\nic_mode_amp=0.005\n", None, True),
    # grain-size rheology (grain_damage=1) on a single-level mesh, where the
    # reference's routine is deterministic (the first level visited evolves; it is
    # the only one): cold top (the grain size stays at 1e-3, the clip sets the
    # viscosity near the top) and a warmer top boundary
    "gd_l5": ("level=5\nmg_min_level=4\nmax_timestep=3\ndevelop_mode=0\nRayleigh=1e5\nA=0.0\n"
              "ic_kind=1\nic_seed=42\nic_noise=1e-4\nT_mantle_perturb=0.01\nT_wave_number=1\n"
              "grain_damage=1\nlowest_vis=1e-3\nhighest_vis=1e3\n", None, True),
    "gdw_l5": ("level=5\nmg_min_level=4\nmax_timestep=2\ndevelop_mode=0\nRayleigh=1e5\nA=2.0\n"
               "ic_kind=1\nic_seed=42\nic_noise=1e-4\nT_mantle_perturb=0.01\nT_wave_number=1\n"
               "top_T_bc_val=0.5\ngrain_damage=1\nlowest_vis=1e-3\nhighest_vis=1e3\n", None, True),
}


TEXT_CASES = {"cfg1_l5"}   # cases whose Output.c text files are kept too


def run_case(name, extra, keep_steps, keep_coarse):
    text = BASE + extra
    work = tempfile.mkdtemp(prefix="mclg_golden_")
    try:
        inp = os.path.join(work, "case.input")
        with open(inp, "w") as fh:
            fh.write(text)
        dump = os.path.join(work, "dump")
        os.makedirs(dump)
        env = dict(os.environ, MCLG_DUMP_DIR=dump)
        if name in TEXT_CASES:
            env["MCLG_REF_TEXT"] = "1"   # the harness also calls the reference's own output()
        proc = subprocess.run([REF_BIN, inp], cwd=work, env=env, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"{name}: reference exited {proc.returncode}\n{proc.stderr[-2000:]}")
        out = {}
        if name in TEXT_CASES:   # Output.c files, verbatim
            for root, _, files in os.walk(os.path.join(work, "out")):
                for f in files:
                    rel_path = os.path.relpath(os.path.join(root, f), os.path.join(work, "out"))
                    with open(os.path.join(root, f), "rb") as fh:
                        out["text/" + rel_path] = np.frombuffer(fh.read(), np.uint8)
        uz = [int(m.group(1)) for m in re.finditer(r"^(\d+) dv = ", proc.stdout, re.M)]
        heat = [int(m.group(1)) for m in re.finditer(r"Temperature CG cycle = (\d+)", proc.stdout)]
        mesh = read_dump(os.path.join(dump, "mesh.dump"))
        fine = int(mesh["levels"][1]) - 1
        for k, v in mesh.items():
            if keep_coarse or "@" not in k or k.endswith(f"@{fine}"):
                out["mesh/" + k] = v
        ops = read_dump(os.path.join(dump, "stokes_ops.dump"))
        for k, v in ops.items():
            if keep_coarse or k.endswith(f"@{fine}"):
                out["ops/" + k] = v
        steps = sorted(int(f[5:12]) for f in os.listdir(dump) if f.startswith("step_"))
        series = {"dt": [], "model_time": [], "res_m": [], "res_c": []}
        for s in steps:
            st = read_dump(os.path.join(dump, f"step_{s:07d}.dump"))
            ht = read_dump(os.path.join(dump, f"heat_{s:07d}.dump"))
            r = st["residual"]
            series["res_m"].append(r[0] / r[2])
            series["res_c"].append(r[1] / r[2])
            series["dt"].append(float(ht["dt"][0]))
            series["model_time"].append(float(ht["model_time"][0]))
            if keep_steps is None or s in keep_steps:
                for k, v in st.items():
                    out[f"step{s:04d}/{k}"] = v
                for k, v in ht.items():
                    out[f"heat{s:04d}/{k}"] = v
        for k, v in series.items():
            out["series/" + k] = np.asarray(v)
        out["series/uzawa_cycles"] = np.asarray(uz, np.int32)
        out["series/heat_cg_cycles"] = np.asarray(heat, np.int32)
        out["series/steps"] = np.asarray(steps, np.int32)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        with open(os.path.join(HERE, f"{name}.input"), "w") as fh:
            fh.write(text)
        print(f"{name}: {len(steps)} steps, uzawa cycles {uz[:6]}..., "
              f"{os.path.getsize(os.path.join(HERE, name + '.npz')) / 1e6:.2f} MB")
    finally:
        shutil.rmtree(work, ignore_errors=True)


def main(argv):
    if not os.path.exists(REF_BIN):
        sys.exit(f"{REF_BIN} missing: run make -C oracle/ref first")
    names = argv[1:] or list(CASES)
    for n in names:
        run_case(n, *CASES[n])


if __name__ == "__main__":
    main(sys.argv)
