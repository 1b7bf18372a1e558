#!/usr/bin/env python3
"""Time steps per second of the mantle-convection time-step path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl gb300|reference]

A step is one pass of the reference's per-step sequence (Main.c:58-64):
buoyancy, viscosity, K/F/G assembly, the Stokes solve, stress, and the SUPG
temperature update, on seeded synthetic .input workloads
(mantle_convection_lab_gb300/configs).

Default workload -- configuration 3: 1024 x 1024 uniform Q1/P0 mesh, Ra=1e8,
eta = exp(-ln(1e5) T) clipped to [1e-5, 1], every step solved to a true
Stokes residual |[F - K d - G p; G^T d]|/|F| < 1e-8.
  value      steps/s of the mixed-precision solver (FP64 iterative refinement
             around MINRES on the full Stokes system, preconditioned by one FP32
             multigrid V-cycle and the BAB pressure diagonal) with the learned
             guess: each step starts from the linear
             extrapolation of the last two solutions, corrected by the CNN
             (mantle_convection_lab_gb300/weights) when that lowers the FP64
             residual; device time (CUDA events on the engine's stream), fields
             resident in HBM, working set larger than L2 is not guaranteed so
             L2 is flushed (256 MB write) between steps
  mixed_no_network  the same solver and warm start without the network
  plain_fp64 the same solve with FP64 inner solves and the reference's start
             (d = 0, p kept: initial_d_p, Solver.c:251-278)
  e2e        steps/s through mclg_step_host: T copied in from pinned host memory
             and T, V, P copied back every step
  roofline   the persistent Stokes kernel: algorithmic bytes per launch (per-pass
             byte counts x measured iteration counts) / its CUDA-event duration,
             against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (a restatement of the reference's algorithm that
             reproduces it bit for bit) timed on this host's cores on a bounded sample

Under torchrun every rank runs an independent replica (one model per GPU:
the single-model path does not shard) and value is the sum over ranks.
--impl reference times the reference's own CPU algorithm (the oracle).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "cfg3_mg_1024": {
        "input": "mantle_convection_lab_gb300/configs/cfg3_mg_1024.input",
        "kind": "converged",
        "desc": "configuration 3: 1024x1024 uniform Q1/P0, Ra=1e8, eta=exp(-ln(1e5) T) in [1e-5,1], "
                "tanh boundary layers + 8 seeded modes, free slip; true Stokes residual < 1e-8 every step",
        "mesh": "1024x1024",
    },
    "cfg1_plain_64": {
        "input": "mantle_convection_lab_gb300/configs/cfg1_plain_64.input",
        "kind": "replica",
        "desc": "configuration 1: 64x64 uniform Q1/P0, Ra=1e5, isoviscous, free slip, FP64 Uzawa + "
                "Jacobi-PCG (the reference's iteration), true Stokes residual < 1e-8",
        "mesh": "64x64",
    },
}
WORKLOADS["cfg4_ensemble_256"] = {
    "input": "mantle_convection_lab_gb300/configs/cfg3_mg_1024.input",
    "kind": "ensemble",
    "desc": "configuration 4: 256 independent models, elements per side from {32,64,128,256}, Ra log-uniform "
            "[1e5,1e7], viscosity contrast log-uniform [1,1e4], seeded perturbations, uniform meshes; mixed "
            "precision, every model to Stokes residual < 1e-8 every step; one batched solver launch per step",
    "mesh": "256 models, 32^2..256^2",
}
WORKLOADS["cfg4_ensemble_amr_256"] = {
    "input": "mantle_convection_lab_gb300/configs/cfg3_mg_1024.input",
    "kind": "ensemble", "amr": True,
    "desc": "configuration 4 with refinement: the 256 members of cfg4_ensemble_256 starting from tanh boundary "
            "layers with seeded modes, each base grid refined 0-2 levels (seeded) by |grad T| > 0.2 max (2:1, "
            "hanging nodes); uniform members in one batched launch, refined members in one batched launch of the "
            "refined-mesh solver; every member to Stokes residual < 1e-8 every step",
    "mesh": "256 models, 32^2..256^2 bases + 0-2 levels",
}
WORKLOADS["cfg2_amr_128"] = {
    "input": "mantle_convection_lab_gb300/configs/cfg2_amr_128.input",
    "kind": "amr",
    "desc": "configuration 2: 128x128 base, |grad T| > 0.2 max refined up to 3 levels (2:1 balanced, hanging "
            "nodes), remeshing every 10 steps, eta=exp(-ln(1e4) T), Ra=1e7; FP32 V-cycle inside FP64 refinement "
            "(MINRES on the conforming hanging-node system) to Stokes residual 1e-8 every step; the FP64 replica "
            "of the reference's Uzawa/Jacobi-PCG iteration beside it",
    "mesh": "128^2 base + 3 levels",
}
ENSEMBLE_METRIC = "aggregate model-steps/s at Stokes residual 1e-8"
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one steady launch
# of the workload's solver kernel, from the ncu capture summarised in profiles/
TRAFFIC = {"cfg3_mg_1024": (45.78e9, "profiles/k_stokes_mg_f32_1024.md (one steady launch, ncu --set full)")}
DEFAULT_WORKLOAD = "cfg3_mg_1024"
GUESS_NET = os.path.join(ROOT, "mantle_convection_lab_gb300", "weights", "guess_cfg3.bin")
GUESS_GRID = 128
METRIC = "time steps/s at Stokes residual 1e-8"


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.fh = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.fh.seek(0)
        rows = [r.split(",") for r in self.fh.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.fh.name)

        def num(s):
            try:
                return float(s)
            except ValueError:
                return None
        sm = [x for x in (num(r[1]) for r in rows) if x is not None]
        mx = [x for x in (num(r[2]) for r in rows) if x is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def replica_bytes(st, neq, nno, nel, w=8):
    """FP64 replica: per inner CG iteration w*(10 n_v + nn) + nn, per Uzawa iteration
    w*(4 n_v + 8 ne), plus the two residual passes around the solve."""
    return (st.cg_cycles * (w * (10 * neq + nno) + nno) + st.uzawa_cycles * w * (4 * neq + 8 * nel)
            + 2 * (w * (10 * neq + nno) + nno))


def converged_bytes(st, N, method=0, w=4, cheb=False, nu=2, nu_c=2, lfine=2):
    """Mixed solver, per launch.  V-cycle: 2 nu tile passes per level (nu sweeps
    per side: nu on the lfine finest levels, nu_c below; read x, b, D^-1 as 2w
    each, eta w, mask 1; write 2w: 9w+1 B/node) and the transfer (restriction
    reads 9 fine residuals per coarse node, prolongation 4 coarse values per fine
    node, cached: counted as 4w B per fine node); the Chebyshev pairs (levels
    with 2 sweeps) also write and read back the coarse-corrected iterate on the
    way up (4w B/node).
    Uzawa (method 0), per inner MG-PCG iteration: the CG part w*(10 n_v + nn) +
    nn plus a V-cycle; per Uzawa iteration: FP64 G s, G^T u and the pressure
    updates, 8*(4 n_v + 8 ne).
    MINRES (method 1), per iteration: a V-cycle, the TI operator (5w+1 B/node),
    and the FP64 Lanczos, direction and solution updates with G and G^T:
    (225 + 10w) B per node and 136 B per element.
    Per refinement pass: FP64 K d + G p residual, 8*(3 n_v + nn) + 8*3 ne."""
    nn = (N + 1) ** 2
    nv = 2 * nn
    ne = N * N
    vcyc, n, lev = 0, N, 0
    while n >= 4:
        m = (n + 1) ** 2
        sweeps = nu if lev < lfine else nu_c
        vcyc += 2 * sweeps * (9 * w + 1) * m + 4 * w * m + (4 * w * m if cheb and sweeps == 2 else 0)
        n //= 2
        lev += 1
    refine = 8 * (3 * nv + nn) + 8 * 3 * ne
    if method == 1:
        it = vcyc + (5 * w + 1) * nn + (225 + 10 * w) * nn + 136 * ne
        extra_vcycles = max(st.cg_cycles - st.uzawa_cycles, 0)
        return st.uzawa_cycles * it + extra_vcycles * (vcyc + 24 * nn) + max(st.refine_passes, 1) * refine
    inner = w * (10 * nv + nn) + nn + vcyc
    outer = 8 * (4 * nv + 8 * ne)
    return st.cg_cycles * inner + st.uzawa_cycles * outer + max(st.refine_passes, 1) * refine


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def init_dist(world, local_rank):
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local_rank)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return dist


def reduce_op(dist, v, op):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=op(dist))
    return float(t.item())


def rmax(dist, v):
    return reduce_op(dist, v, lambda d: d.ReduceOp.MAX)


def rsum(dist, v):
    return reduce_op(dist, v, lambda d: d.ReduceOp.SUM)


def gather_members(dist, local):
    """Per-member results of every rank ({member index: value}) gathered on the
    host of every rank, keyed by member index.  Members are independent, so
    this gather at the end of a run is the only exchange between ranks."""
    if dist is None:
        return dict(local)
    objs = [None] * dist.get_world_size()
    dist.all_gather_object(objs, dict(local))
    out = {}
    for o in objs:
        if set(o) & set(out):
            raise RuntimeError("a member was stepped on two ranks")
        out.update(o)
    return out


def job_throughput(dist, units, seconds):
    """Whole-job rate over independent replicas: the units all ranks processed
    divided by the slowest rank's time."""
    return rsum(dist, units) / rmax(dist, seconds)


# ---- the reference's algorithm on the host cores (the CPU oracle) ---------------
# Everything here runs oracle/ with its own .input reader and uniform mesh
# (oracle/mesh_oracle.py): nothing of the engine is loaded in these arms.
REF_RECORD = os.path.join(ROOT, "oracle", "ref_steps_cfg3_mg_1024.json")


def _oracle_mod():
    p = os.path.join(ROOT, "oracle")
    if p not in sys.path:
        sys.path.insert(0, p)
    import mesh_oracle
    import oracle_port
    return oracle_port, mesh_oracle


def _oracle(inp, threads, mesh_level=None, cfg=None):
    oracle_port, mesh_oracle = _oracle_mod()
    cfg = cfg if cfg is not None else mesh_oracle.read_input(os.path.join(ROOT, inp))
    return oracle_port.Oracle(cfg, threads=threads, standalone=True, mesh_level=mesh_level)


def reference_record():
    """Whole steps of the reference's algorithm on configuration 3 at 1024^2,
    measured by oracle/time_reference_steps.py (per step: Uzawa cycles, inner
    CG iterations, wall time and the host they ran on)."""
    with open(REF_RECORD) as fh:
        return json.load(fh)


def cpu_sample(wl, threads, samples=3, warmup=0, cycles=1):
    """Returns (steps_per_s, cores, description, timed_seconds).

    Configuration 1: whole steps of the reference algorithm.
    Configuration 3 (1024^2): one whole reference step takes minutes (its first
    step runs Uzawa to max_citcom_cycle with every inner CG at max_cg_cycle), so
    each sample is a real step truncated after `cycles` Uzawa cycles -- the
    assembly, the initial inner CG solve, `cycles` Uzawa cycles with their full
    inner solves, the temperature update -- and the whole steps are rebuilt from
    the timed parts and the inner-CG iteration counts of whole reference steps
    recorded in oracle/ref_steps_cfg3_mg_1024.json:
        t_step = t_assembly + t_heat + C_step * (t_solve / C_sample)."""
    if wl["kind"] == "replica":
        o = _oracle(wl["input"], 1)
        for _ in range(max(warmup, 1)):
            o.step()
        t0 = time.perf_counter()
        for _ in range(samples):
            o.step()
        el = time.perf_counter() - t0
        o.close()
        return samples / el, 1, f"{samples} whole steps of the reference algorithm on 1 core ({el:.1f} s)", el
    rec = reference_record()
    o = _oracle(wl["input"], threads)
    t_asm, t_heat, t_cg, timed = [], [], [], 0.0
    for k in range(warmup + samples):
        o.set_caps(cycles, o.cfg.max_cg_cycle)
        t0 = time.perf_counter()
        st = o.step()
        el = time.perf_counter() - t0
        if k >= warmup:
            timed += el
            t_asm.append(st["s_assembly"])
            t_heat.append(st["s_heat"])
            t_cg.append(st["s_solve"] / max(st["cg_cycles"], 1))
    o.close()
    a, h, c = statistics.median(t_asm), statistics.median(t_heat), statistics.median(t_cg)
    steps = rec["steps"]
    total = sum(a + h + s["cg_iterations"] * c for s in steps)
    v = len(steps) / total
    desc = (f"{samples} real steps truncated after {cycles} Uzawa cycle(s) on the 1024^2 mesh with {threads} threads "
            f"(assembly {a:.2f} s, temperature update {h:.2f} s, {1e3 * c:.2f} ms per inner CG iteration), rebuilt "
            f"into the reference's first {len(steps)} whole steps with their recorded inner-CG counts "
            f"{[s['cg_iterations'] for s in steps]} (Uzawa cycles {[s['uzawa_cycles'] for s in steps]}; "
            f"oracle/ref_steps_cfg3_mg_1024.json, whole steps timed on {rec.get('host', 'a host')} with "
            f"{rec['threads']} threads: {[round(s['wall_s'], 1) for s in steps]} s)")
    return v, threads, desc, timed


def _member_config(n_side, rayleigh, contrast, seed):
    """ensemble.member_config on the oracle's own input reader."""
    import math
    _, mesh_oracle = _oracle_mod()
    c = mesh_oracle.read_input(os.path.join(ROOT, "mantle_convection_lab_gb300", "configs", "cfg3_mg_1024.input"))
    c.level = int(round(math.log2(n_side))) + 1
    c.mg_min_level = 1
    c.Rayleigh, c.A, c.refT = rayleigh, math.log(contrast), 0.0
    c.vis_min, c.vis_max = 1.0 / contrast, 1.0
    c.ic_kind, c.ic_seed, c.ic_noise, c.T_mantle_perturb, c.T_wave_number = 1, seed, 1e-3, 0.01, 1
    return c


def ensemble_cpu_sample(threads, steps=2):
    """The reference's algorithm on one member of each size class (its first
    member in the draw), `steps` whole steps each with all threads; the
    ensemble's rate rebuilt as 256 / sum over members of the measured step time
    of the member's size class."""
    from mantle_convection_lab_gb300 import ensemble   # the draw only (numpy)
    params = ensemble.draw(256, 4)
    per = {}
    timed = 0.0
    for side in ensemble.SIZES:
        p = next(q for q in params if q[0] == side)
        o = _oracle(None, threads, cfg=_member_config(*p))
        t0 = time.perf_counter()
        for _ in range(steps):
            o.step()
        el = time.perf_counter() - t0
        o.close()
        timed += el
        per[side] = el / steps
    total = sum(per[q[0]] for q in params)
    return 256 / total, threads, (f"{steps} whole steps of the reference algorithm on one member per size class with "
                                  f"{threads} threads (s/step: " + ", ".join(f"{k}^2 {v:.2f}" for k, v in per.items())
                                  + "), the 256-member mix rebuilt from the per-class step times"), timed


def _ref_line(args, world, metric, v, unit, cores, sample, timed, steps, warmup, extra=None):
    line = {"metric": metric, "impl": "reference", "value": v, "unit": unit, "n_gpus": world, "steps": steps,
            "warmup": warmup, "ms_per_step": 1e3 / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded .input)",
            "config": {"workload": args.workload, "desc": WORKLOADS[args.workload]["desc"],
                       "mesh": WORKLOADS[args.workload]["mesh"]},
            "cpu_baseline": {"value": v, "unit": unit, "cores": cores, "kind": "port", "sample": sample},
            "timed_s": timed,
            "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if extra:
        line.update(extra)
    print(json.dumps(line), flush=True)


def run_reference(args, wl):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    if wl["kind"] == "amr":
        _, mesh_oracle = _oracle_mod()
        cfg = mesh_oracle.read_input(os.path.join(ROOT, wl["input"]))
        cfg.max_citcom_cycle, cfg.max_cg_cycle = 200, 500
        o = _oracle(None, threads, mesh_level=8, cfg=cfg)   # the unrefined 128 x 128 base
        t0 = time.perf_counter()
        o.step()
        el = time.perf_counter() - t0
        o.close()
        _ref_line(args, world, "time steps/s including remeshing (configuration 2)", 1.0 / el, "steps/s", threads,
                  f"one whole step of the reference's algorithm (caps 200 x 500) on the unrefined 128x128 base mesh "
                  f"with {threads} threads: a lower bound on a refined step's cost", el, 1, 0)
        return 0
    if wl["kind"] == "ensemble":
        v, cores, sample, timed = ensemble_cpu_sample(threads)
        _ref_line(args, world, ENSEMBLE_METRIC, v, "model-steps/s", cores, sample, timed, args.steps, args.warmup)
        return 0
    if wl["kind"] == "replica":
        v, cores, sample, timed = cpu_sample(wl, threads, samples=max(1, args.steps), warmup=max(0, args.warmup))
        _ref_line(args, world, METRIC, v, "steps/s", cores, sample, timed, max(1, args.steps), args.warmup)
        return 0
    # configuration 3: bounded samples of real steps, rebuilt with recorded whole-step counts
    n = max(1, min(args.steps, 10))
    v, cores, sample, timed = cpu_sample(wl, threads, samples=n, warmup=1 if args.warmup > 0 else 0)
    rec = reference_record()
    _ref_line(args, world, METRIC, v, "steps/s", cores, sample, timed, n, 1 if args.warmup > 0 else 0,
              {"extrapolated": "whole steps rebuilt from timed parts and recorded iteration counts",
               "reference_residual": "the reference stops on its own update-size test "
                                     "(citcom_solver_accu, Solver.c:131); its Stokes residual after a step is "
                                     + ", ".join(f"{max(s['res_momentum'], s['res_continuity']):.2g}"
                                                 for s in rec["steps"]) + ", never 1e-8"})
    return 0


# ---- FP64 parity of the mixed-precision solvers ----------------------------------
PARITY_RTOL = 1e-12


def fp64_reference_config(cfg):
    """A copy of `cfg` for the FP64 oracle solve of a step: FP64 operator and
    multigrid (precision fp64mg), MINRES, cold start, residual 1e-12."""
    from mantle_convection_lab_gb300 import Config
    c = Config()
    C_ = __import__("ctypes")
    C_.memmove(C_.byref(c), C_.byref(cfg), C_.sizeof(Config))
    c.precision, c.stokes_method, c.warm_start = 2, 1, 0
    c.stokes_rtol, c.outer_rtol, c.max_refine, c.max_outer = PARITY_RTOL, 1e-3, 80, 4000
    return c


def leaves_of(model, cfg):
    """Finest-level Morton start codes of a model's current leaves: its Mcode
    list without the level bits."""
    import numpy as np
    return np.ascontiguousarray(model.mesh("Mcode") >> 4, np.int32)


def _rel(a, b):
    import numpy as np
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b)) / (nb if nb > 0 else 1.0)


def step_parity(model, cfg, leaves=None, step=None):
    """Errors of one mixed-precision step against an FP64 solution of the same
    step: both start from the model's current temperature; the FP64 model
    solves to residual 1e-12 (fp64mg, whose solutions are pinned to the
    reference's fixtures).  Returns relative L2 errors of V (both components),
    P (mean removed: the constant is the null mode of G on the free-slip box)
    and T after the step.  `step` steps the mixed model (default model.step)."""
    from mantle_convection_lab_gb300 import Model
    T0 = model.get("T")
    st = (step or model.step)()
    mine = {k: model.get(k) for k in ("V0", "V1", "P", "T")}
    with Model(fp64_reference_config(cfg), leaves=leaves) as ref:
        ref.set("T", T0)
        rs = ref.step()
        theirs = {k: ref.get(k) for k in ("V0", "V1", "P", "T")}
    import numpy as np
    V = _rel(np.concatenate([mine["V0"], mine["V1"]]), np.concatenate([theirs["V0"], theirs["V1"]]))
    P = _rel(mine["P"] - mine["P"].mean(), theirs["P"] - theirs["P"].mean())
    return {"V": V, "P": P, "T": _rel(mine["T"], theirs["T"]),
            "mixed_residual": max(st.res_momentum, st.res_continuity) if st is not None else None,
            "fp64_residual": max(rs.res_momentum, rs.res_continuity)}


# ---- GPU arm --------------------------------------------------------------------
def timed_steps(model, steps, flush, torch):
    acc = {"ms_total": 0.0, "ms_solver": 0.0, "launches": 0, "uz": 0, "cg": 0, "refine": 0, "res": 0.0,
           "stats": []}
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        st = model.step()
        acc["ms_total"] += st.ms_total
        acc["ms_solver"] += st.solver_kernel_ms
        acc["launches"] += st.kernel_launches
        acc["uz"] += st.uzawa_cycles
        acc["cg"] += st.cg_cycles
        acc["refine"] += st.refine_passes
        acc["res"] = max(acc["res"], st.res_momentum, st.res_continuity)
        acc["stats"].append(st)
    return acc


def attach_guess(model, wl, args):
    """The learned initial guess (converged workloads with trained weights)."""
    from mantle_convection_lab_gb300 import Cnn
    from mantle_convection_lab_gb300.api import GUESS_LEARNED
    if wl["kind"] != "converged" or args.no_learned or not os.path.exists(GUESS_NET):
        return None
    net = Cnn.load(GUESS_NET)
    model.guess_set(GUESS_LEARNED, GUESS_GRID, net)
    return net


def run_ensemble(args, wl):
    import torch
    from mantle_convection_lab_gb300 import ensemble

    rank, world, local_rank = dist_env()
    dist = init_dist(world, local_rank)
    torch.cuda.set_device(local_rank)
    amr_run = wl.get("amr", False)
    # the 256 members are sharded over the ranks (rank r: members r, r + N, ...)
    mine = ensemble.shard(256, rank, world)
    e = ensemble.make_amr(256, seed=4, members=mine) if amr_run else ensemble.make(256, seed=4, members=mine)
    n = e.n
    levels = ensemble.amr_levels(256, 4) if amr_run else None
    # the cluster-size autotuner times one candidate on each of steps 2..6:
    # warm up past it so that the timed steps use its choice
    warmup = max(args.warmup, 7)
    for _ in range(warmup):
        e.step()
    sampler = ClockSampler() if rank == 0 else None
    if sampler:
        sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ms, ms_solver, launches, res, inner = 0.0, 0.0, 0, 0.0, 0
    grids, graph_used = [], False
    # one loop for both figures, so that they cover the same steps: value from the
    # device time of each step (CUDA events), e2e from the wall clock of the same
    # step followed by every member's temperature read back to the host
    wall, d2h = 0.0, 0
    member_res = [0.0] * n
    for _ in range(args.steps):
        t0 = time.perf_counter()
        st = e.step()
        for m in e.members:
            d2h += 8 * m.get("T").size
        wall += time.perf_counter() - t0
        ms += st[0].ms_total
        ms_solver += st[0].solver_kernel_ms
        launches += st[0].kernel_launches
        for k, s_ in enumerate(st):
            member_res[k] = max(member_res[k], s_.res_momentum, s_.res_continuity)
        res = max(res, max(max(s.res_momentum, s.res_continuity) for s in st))
        inner += sum(s.cg_cycles for s in st)
        assert all(s.status == 0 for s in st), [s.status for s in st]
        grids.append(e.cluster_used)
        graph_used = e.graph
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop() if sampler else None
    value = job_throughput(dist, n * args.steps, ms / 1e3)
    e2e = job_throughput(dist, n * args.steps, wall)
    # per-member results gathered on the host: final temperature checksum, residual
    done = gather_members(dist, {i: (float(m.get("T").sum()), float(member_res[k]))
                                 for k, (i, m) in enumerate(zip(mine, e.members))})
    res = max(v[1] for v in done.values())
    # FP64 parity: one more ensemble step; the first member of each size class
    # (and refinement depth) on this rank against its own FP64 solution
    picks, seen = [], set()
    params = ensemble.draw(256, 4)
    for k, i in enumerate(mine):
        key = (params[i][0], int(levels[i]) if levels is not None else 0)
        if key not in seen:
            seen.add(key)
            picks.append(k)
    picks = picks[:6]
    cfgs = ensemble.amr_configs(256, 4, members=[mine[k] for k in picks]) if amr_run else \
        ensemble.configs(256, 4, members=[mine[k] for k in picks])
    T0 = {k: e.members[k].get("T") for k in picks}
    e.step()
    member_parity = []
    for k, cfg_k in zip(picks, cfgs):
        m = e.members[k]
        mine_f = {f: m.get(f) for f in ("V0", "V1", "P", "T")}
        from mantle_convection_lab_gb300 import Model
        import numpy as np
        lv = None
        if amr_run:   # a refined member's configuration names its base grid; its tree is levels deeper
            cfg_k.level += int(levels[mine[k]])
            lv = leaves_of(m, cfg_k)
        with Model(fp64_reference_config(cfg_k), leaves=lv) as ref:
            ref.set("T", T0[k])
            rs = ref.step()
            th = {f: ref.get(f) for f in ("V0", "V1", "P", "T")}
        member_parity.append({
            "member": mine[k], "elements_per_side": params[mine[k]][0],
            "refinement_levels": int(levels[mine[k]]) if levels is not None else 0,
            "V": _rel(np.concatenate([mine_f["V0"], mine_f["V1"]]), np.concatenate([th["V0"], th["V1"]])),
            "P": _rel(mine_f["P"] - mine_f["P"].mean(), th["P"] - th["P"].mean()),
            "T": _rel(mine_f["T"], th["T"]), "fp64_residual": max(rs.res_momentum, rs.res_continuity)})
    sizes = [p[0] for p in ensemble.draw(256, 4)]
    # algorithmic bytes of the batched solver launch: the per-model MINRES model, summed
    line = {
        "metric": ENSEMBLE_METRIC, "value": value, "unit": "model-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32 inner / f64 outer", "data": "synthetic (seeded members)",
        "config": {"workload": args.workload, "desc": wl["desc"], "mesh": wl["mesh"],
                   "members_by_size": {str(k): sizes.count(k) for k in ensemble.SIZES},
                   "members_by_refinement_levels": ({str(k): int((levels == k).sum()) for k in (0, 1, 2)}
                                                    if levels is not None else {"0": n}),
                   "parallelism": f"members sharded over {world} rank(s), rank r steps members r, r+{world}, ...",
                   "members_this_rank": n, "members_gathered": len(done),
                   "l2": "working set > L2 (256 models)",
                   "solver_ms_per_step": ms_solver / args.steps if ms_solver > 0 else None,
                   "step_graph": graph_used, "cluster_size_per_step": grids,
                   "inner_per_model_step": inner / (n * args.steps), "max_stokes_residual": res},
        "e2e": {"value": e2e, "unit": "model-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": d2h // max(args.steps, 1)},
        "gpu_launches": launches,
        "roofline": None,
        "clocks": clocks,
        "parity": {"members": member_parity,
                   "max": {f: max(p[f] for p in member_parity) for f in ("V", "P", "T")},
                   "against": "one more ensemble step; each listed member's step from the same temperature solved "
                              "alone in FP64 (fp64mg, MINRES) to residual 1e-12; relative L2, pressure mean-free"},
    }
    e.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, sample, _ = ensemble_cpu_sample(os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": v, "unit": "model-steps/s", "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def _amr_arm(cfg, steps, warmup, sampler_on, dist, torch, lag=0, parity=False):
    import numpy as np
    from mantle_convection_lab_gb300 import amr
    run = amr.AmrRun(cfg, lag=lag)
    for _ in range(max(warmup, 0)):
        run.step()
    sampler = ClockSampler() if sampler_on else None
    if sampler:
        sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    acc = {"ms": 0.0, "ms_solver": 0.0, "res": 0.0, "nel": [], "launches": 0, "capped": 0, "passes": 0,
           "minres": 0, "vcycles": 0, "rem0": run.remeshes}
    for _ in range(steps):
        st = run.step()
        acc["ms"] += st.ms_total
        acc["ms_solver"] += st.solver_kernel_ms
        acc["launches"] += st.kernel_launches
        acc["res"] = max(acc["res"], st.res_momentum, st.res_continuity)
        acc["capped"] += st.status == 1
        acc["passes"] += st.refine_passes
        acc["minres"] += st.uzawa_cycles
        acc["vcycles"] += st.cg_cycles
        acc["nel"].append(run.model.nel)
        acc["remesh_ms"] = {k: round(getattr(st, "remesh_ms_" + k), 2)
                            for k in ("numbering", "lists", "state", "wait", "carry")}
    torch.cuda.synchronize()
    acc["wall"] = time.perf_counter() - t0
    if dist:
        dist.barrier()
    acc["clocks"] = sampler.stop() if sampler else None
    acc["remeshes"] = run.remeshes - acc["rem0"]
    acc["nh"] = run.model.nh
    acc["ms_remesh_begin"] = float(np.mean(run.ms_begin)) if run.ms_begin else None
    acc["ms_remesh_end"] = float(np.mean(run.ms_end)) if run.ms_end else None
    if parity:
        # one more step on the current refined mesh against its FP64 solution
        acc["parity"] = step_parity(run.model, cfg, leaves=leaves_of(run.model, cfg))
    run.close()
    return acc


def run_amr(args, wl):
    """Configuration 2: steps including the remeshing every 10 steps (host tree
    and transfer, device flags), timed on the wall clock because remeshing is
    host work; the device time of the steps is reported beside it.  value: the
    mixed-precision converged solver (FP64 refinement around MINRES with an FP32
    V-cycle on the mesh's own levels, conforming hanging-node space) to Stokes
    residual 1e-8; fp64_replica: the reference's iteration (Uzawa + Jacobi-PCG)
    on the same run with bounded caps, which does not converge here."""
    import torch
    from mantle_convection_lab_gb300 import Config

    rank, world, local_rank = dist_env()
    dist = init_dist(world, local_rank)
    torch.cuda.set_device(local_rank)
    cfg = Config.from_input(os.path.join(ROOT, wl["input"]))
    cfg.precision, cfg.warm_start, cfg.stokes_method, cfg.stokes_rtol = 1, 3, 1, 1e-8
    cfg.outer_rtol, cfg.max_outer, cfg.max_refine = 1e-2, 1000, 20
    cfg.mg_smooth = 1          # one Jacobi sweep per side: fewest grid barriers per V-cycle
    cfg.mg_eta_avg = 1         # coarse viscosity: full-weighted mean (fewest MINRES iterations here)
    # remeshes after the first are asynchronous: the new mesh is built on a host
    # thread during the next two steps, which run on the old mesh
    acc = _amr_arm(cfg, args.steps, args.warmup, rank == 0, dist, torch, lag=2, parity=True)
    value = job_throughput(dist, args.steps, acc["wall"])
    line = {
        "metric": "time steps/s including remeshing at Stokes residual 1e-8 (configuration 2)", "value": value,
        "unit": "steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * acc["wall"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 inner / f64 outer", "data": "synthetic (seeded .input)",
        "config": {"workload": args.workload, "desc": wl["desc"], "mesh": wl["mesh"],
                   "elements_per_step": acc["nel"], "hanging_nodes_last": acc["nh"],
                   "remeshes_timed": acc["remeshes"], "device_ms_per_step": acc["ms"] / args.steps,
                   "ms_per_remesh_begin": acc["ms_remesh_begin"], "ms_per_remesh_end": acc["ms_remesh_end"],
                   "last_remesh_ms": acc.get("remesh_ms"),
                   "solver_kernel_ms_per_step": acc["ms_solver"] / args.steps,
                   "refine_passes_per_step": acc["passes"] / args.steps,
                   "minres_iterations_per_step": acc["minres"] / args.steps,
                   "steps_at_iteration_cap": acc["capped"], "max_stokes_residual": acc["res"],
                   "residual": "conforming: |[C^T(F - K d - G p); G^T C d]| / |C^T F|, C the hanging-node expansion",
                   "residual_1e-8_met": bool(acc["res"] < 1e-8), "parallelism": f"replicas x{world}",
                   "remesh": "every 10 steps from the T of that step: flags, tree and numbering on the device, "
                             "the solver's lists and the new device state built on a host thread during the next "
                             "2 steps, swapped in before the third",
                   "roofline": "not reported: assembled-ELL operators on 5 levels, latency-bound at this size"},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": acc["launches"], "roofline": None, "clocks": acc["clocks"],
        "parity": dict(acc["parity"], against="one more step on the last refined mesh from the same temperature, "
                       "solved in FP64 (fp64mg, MINRES on the conforming system) to residual 1e-12; relative L2, "
                       "pressure mean-free"),
    }
    if not args.no_plain:
        rcfg = Config.from_input(os.path.join(ROOT, wl["input"]))
        rcfg.max_citcom_cycle, rcfg.max_cg_cycle = 200, 500
        n = min(args.plain_steps, args.steps)
        racc = _amr_arm(rcfg, n, 1, False, dist, torch)
        line["fp64_replica"] = {
            "value": job_throughput(dist, n, racc["wall"]), "unit": "steps/s", "steps": n,
            "max_stokes_residual": racc["res"], "steps_at_iteration_cap": racc["capped"],
            "desc": "the reference's iteration (BAB-multiply Uzawa, Jacobi-PCG, hanging nodes overwritten in CG) "
                    "in FP64 with caps 200 x 500; it does not reach the residual on this mesh"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def run_gpu(args, wl):
    import torch
    from mantle_convection_lab_gb300 import Config, Model

    if wl["kind"] == "ensemble":
        return run_ensemble(args, wl)
    if wl["kind"] == "amr":
        return run_amr(args, wl)

    rank, world, local_rank = dist_env()
    dist = init_dist(world, local_rank)
    torch.cuda.set_device(local_rank)
    cfg = Config.from_input(os.path.join(ROOT, wl["input"]))
    model = Model(cfg)
    model.initial_temperature()
    net = attach_guess(model, wl, args)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    for _ in range(max(args.warmup, 0)):
        model.step()

    sampler = ClockSampler() if rank == 0 else None
    if sampler:
        sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    acc = timed_steps(model, args.steps, flush, torch)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    if dist:
        dist.barrier()
    clocks = sampler.stop() if sampler else None
    value = job_throughput(dist, args.steps, acc["ms_total"] / 1e3)

    # end-to-end through the host-buffer entry point
    nno, nel = model.nno, model.nel
    T_in = torch.empty(nno, dtype=torch.float64, pin_memory=True).numpy()
    T_out = torch.empty(nno, dtype=torch.float64, pin_memory=True).numpy()
    V_out = torch.empty(2 * nno, dtype=torch.float64, pin_memory=True).numpy()
    P_out = torch.empty(nel, dtype=torch.float64, pin_memory=True).numpy()
    T_in[:] = model.get("T")
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        model.step_host(T_in, T_out, V_out, P_out)
        T_in[:] = T_out
    e2e = job_throughput(dist, args.steps, time.perf_counter() - t0)

    peak, peak_kind = load_peaks()
    n_launch = max(len(acc["stats"]), 1)
    if wl["kind"] == "converged":
        nu = max(cfg.mg_smooth, 1)
        alg = sum(converged_bytes(s, cfg_N(cfg), cfg.stokes_method, cheb=cfg.mg_smoother == 1, nu=nu,
                                  nu_c=cfg.mg_smooth_coarse if cfg.mg_smooth_coarse > 0 else nu,
                                  lfine=cfg.mg_fine_levels)
                  for s in acc["stats"]) / n_launch
        kname = "k_stokes_mg<float> (persistent mixed-precision Stokes solve)"
        dtype = "f32 inner / f64 outer"
    else:
        alg = sum(replica_bytes(s, model.neq, nno, nel) for s in acc["stats"]) / n_launch
        kname = "k_uzawa (persistent FP64 Uzawa/CG)"
        dtype = "f64"
    ms_launch = acc["ms_solver"] / n_launch
    achieved = alg / (ms_launch / 1e3) / 1e9 if ms_launch > 0 else 0.0
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": acc["ms_total"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype,
        "data": "synthetic (seeded .input, Philox initial temperature)",
        "config": {"workload": args.workload, "desc": wl["desc"], "mesh": wl["mesh"],
                   "parallelism": f"replicas x{world}", "l2": "flushed (256 MB write) between steps",
                   "outer_iterations_per_step": acc["uz"] / args.steps, "vcycles_or_inner_cg_per_step": acc["cg"] / args.steps,
                   "correction_solve": ["Uzawa + inner MG-PCG", "MINRES, block-diagonal preconditioner"][cfg.stokes_method]
                   if wl["kind"] == "converged" else "Uzawa + Jacobi-PCG (reference iteration)",
                   "refine_passes_per_step": acc["refine"] / args.steps, "max_stokes_residual": acc["res"]},
        "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": 8 * nno,
                "d2h_bytes_per_step": 8 * (3 * nno + nel)},
        "gpu_launches": acc["launches"],
        "roofline": {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": TRAFFIC.get(args.workload, (None, None))[0],
                     "traffic_source": TRAFFIC.get(args.workload, (None, None))[1],
                     "alg_bytes_per_launch": alg, "ms_per_launch": ms_launch},
        "clocks": clocks,
        "wall_s_timed": wall,
    }
    if wl["kind"] == "converged":
        line["parity"] = dict(step_parity(model, cfg), against="the same step from the same temperature solved in "
                              "FP64 (fp64mg, MINRES) to Stokes residual 1e-12; relative L2, pressure mean-free")
    if net is not None:
        line["learned_guess"] = {
            "network": os.path.relpath(GUESS_NET, ROOT), "params": net.nparam, "grid": GUESS_GRID,
            "steps_network_kept": sum(1 for s in acc["stats"] if s.guess_used == 1),
            "steps_judged": sum(1 for s in acc["stats"] if s.guess_used >= 0),
            "ms_guess_per_step": sum(s.ms_guess for s in acc["stats"]) / args.steps,
            "desc": "CNN correction of the extrapolated guess, kept only when its FP64 residual is smaller"}
    model.close()
    del model
    if net is not None and not args.no_plain:
        # the same solver without the network
        mcfg = Config.from_input(os.path.join(ROOT, wl["input"]))
        mm = Model(mcfg)
        mm.initial_temperature()
        for _ in range(max(args.warmup, 0)):
            mm.step()
        torch.cuda.synchronize()
        macc = timed_steps(mm, args.steps, flush, torch)
        mm.close()
        mv = job_throughput(dist, args.steps, macc["ms_total"] / 1e3)
        line["mixed_no_network"] = {"value": mv, "unit": "steps/s", "steps": args.steps,
                                    "ms_per_step": macc["ms_total"] / args.steps,
                                    "uzawa_cycles_per_step": macc["uz"] / args.steps,
                                    "inner_cg_per_step": macc["cg"] / args.steps,
                                    "max_stokes_residual": macc["res"]}
    if wl["kind"] == "converged" and not args.no_plain:
        # FP64 with the same method and warm start as the headline arm: what precision alone buys
        fcfg = Config.from_input(os.path.join(ROOT, wl["input"]))
        fcfg.precision = 2
        fm = Model(fcfg)
        fm.initial_temperature()
        for _ in range(max(args.warmup, 0)):
            fm.step()
        torch.cuda.synchronize()
        facc = timed_steps(fm, args.plain_steps, flush, torch)
        fm.close()
        fv = job_throughput(dist, args.plain_steps, facc["ms_total"] / 1e3)
        line["fp64_minres"] = {"value": fv, "unit": "steps/s", "steps": args.plain_steps,
                               "ms_per_step": facc["ms_total"] / args.plain_steps,
                               "minres_per_step": facc["uz"] / args.plain_steps,
                               "max_stokes_residual": facc["res"],
                               "desc": "FP64 operator and multigrid (fp64mg), MINRES, extrapolated warm start: the "
                                       "headline arm's method without the mixed precision and the network"}
        pcfg = Config.from_input(os.path.join(ROOT, wl["input"]))
        pcfg.precision = 2
        pcfg.warm_start = 2
        pcfg.stokes_method = 0       # Uzawa outer loop with inner MG-PCG, as the reference iterates
        pcfg.outer_rtol = 1e-2
        pcfg.inner_rtol = 1e-2
        pm = Model(pcfg)
        pm.initial_temperature()
        for _ in range(max(args.warmup, 0)):
            pm.step()
        torch.cuda.synchronize()
        pacc = timed_steps(pm, args.plain_steps, flush, torch)
        pm.close()
        pv = job_throughput(dist, args.plain_steps, pacc["ms_total"] / 1e3)
        line["plain_fp64"] = {"value": pv, "unit": "steps/s", "steps": args.plain_steps,
                              "ms_per_step": pacc["ms_total"] / args.plain_steps,
                              "uzawa_cycles_per_step": pacc["uz"] / args.plain_steps,
                              "inner_cg_per_step": pacc["cg"] / args.plain_steps,
                              "max_stokes_residual": pacc["res"],
                              "desc": "the reference's Uzawa outer loop with FP64 multigrid-preconditioned inner CG, "
                                      "d=0 and p kept each step (the reference's start)"}
        line["speedup_vs_plain_fp64"] = value / pv
        best64 = max(pv, fv)
        line["ablation"] = {
            "steps_per_s": {"fp64_uzawa_reference_start": pv, "fp64_minres_extrapolated": fv,
                            "mixed_minres_extrapolated": line.get("mixed_no_network", {}).get("value"),
                            "mixed_minres_extrapolated_learned": value},
            "what_each_buys": {"method_and_warm_start_in_fp64": fv / pv,
                               "mixed_precision": (line["mixed_no_network"]["value"] / fv
                                                   if "mixed_no_network" in line else None),
                               "network": (value / line["mixed_no_network"]["value"]
                                           if "mixed_no_network" in line else None)},
            "headline_vs_strongest_fp64": value / best64}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, sample, _ = cpu_sample(wl, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": v, "unit": "steps/s", "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def cfg_N(cfg):
    return 1 << (cfg.level - 1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_gpu(args, wl)


if __name__ == "__main__":
    sys.exit(main())
