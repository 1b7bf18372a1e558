#!/usr/bin/env python3
"""Time steps per second of the mantle-convection time-step path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl gb300|reference]

A step is one pass of the reference's per-step sequence (Main.c:58-64):
buoyancy, viscosity, K/F/G assembly, the Uzawa Stokes solve to the
configured tolerance, stress, and the SUPG temperature update.  The inputs
are the seeded synthetic .input workloads in mantle_convection_lab_gb300/configs.

One JSON line on rank 0:
  value      steps/s over all ranks, device time (CUDA events on the engine's
             stream), fields resident in HBM, L2 flushed between steps
  e2e        steps/s through mclg_step_host: temperature copied in from pinned
             host memory and T, V, P copied back every step
  roofline   the persistent Stokes solver kernel: algorithmic bytes per launch
             (per-iteration byte counts x measured iteration counts) / its
             CUDA-event duration, against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (a restatement of the reference's algorithm that
             reproduces it bit for bit) timed on this host's cores on a bounded sample

Under torchrun every rank runs an independent replica (the single-model path
does not shard; ensembles shard by model) and value is the sum over ranks.
--impl reference times the reference's CPU algorithm (the oracle) instead.
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
    "cfg1_plain_64": {
        "input": "mantle_convection_lab_gb300/configs/cfg1_plain_64.input",
        "desc": "configuration 1: 64x64 uniform Q1/P0, Ra=1e5, isoviscous, free slip, FP64 Uzawa + "
                "Jacobi-PCG (the reference's iteration), true Stokes residual < 1e-8",
        "mesh": "64x64",
    },
}
DEFAULT_WORKLOAD = "cfg1_plain_64"


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
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def stokes_bytes(st, neq, nno, nel, w=8):
    """Algorithmic bytes of one Stokes solve: per inner CG iteration w*(10 n_v + nn) + nn,
    per Uzawa iteration w*(4 n_v + 8 ne), plus the prologue/epilogue (two residual passes)."""
    cg = st.cg_cycles * (w * (10 * neq + nno) + nno)
    uz = st.uzawa_cycles * w * (4 * neq + 8 * nel)
    pro = 2 * (w * (10 * neq + nno) + nno)
    return cg + uz + pro


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


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def cpu_sample(inp, steps):
    """Time the CPU oracle for `steps` steady steps (after one setup step)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_port
    o = oracle_port.Oracle(os.path.join(ROOT, inp), threads=1)
    o.step()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    dt = time.perf_counter() - t0
    o.close()
    return steps / dt, dt


def run_reference(args, wl):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    steps = max(1, args.steps)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_port
    o = oracle_port.Oracle(os.path.join(ROOT, wl["input"]), threads=1)
    for _ in range(max(0, args.warmup)):
        o.step()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    el = time.perf_counter() - t0
    v = steps / el
    line = {"metric": "time steps/s at Stokes residual 1e-8", "impl": "reference", "value": v,
            "unit": "steps/s", "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded .input)",
            "config": {"workload": args.workload, "desc": wl["desc"]},
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": 1, "kind": "port",
                             "sample": f"{steps} steps of {args.workload} after {args.warmup} warm-up steps"},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, wl):
    import numpy as np
    import torch
    from mantle_convection_lab_gb300 import Config, Model

    rank, world, local_rank = dist_env()
    dist = init_dist(world, local_rank)
    torch.cuda.set_device(local_rank)
    cfg = Config.from_input(os.path.join(ROOT, wl["input"]))
    model = Model(cfg)
    model.initial_temperature()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2
    for _ in range(max(args.warmup, 0)):
        model.step()

    # device-timed region
    sampler = ClockSampler() if rank == 0 else None
    if sampler:
        sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ms_total, ms_solver, launches, alg_bytes, uz, cgc, res = 0.0, 0.0, 0, 0, 0, 0, 0.0
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        st = model.step()
        ms_total += st.ms_total
        ms_solver += st.solver_kernel_ms
        launches += st.kernel_launches
        alg_bytes += stokes_bytes(st, model.neq, model.nno, model.nel)
        uz += st.uzawa_cycles
        cgc += st.cg_cycles
        res = max(res, st.res_momentum, st.res_continuity)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    if dist:
        dist.barrier()
    clocks = sampler.stop() if sampler else None
    t_max = reduce_max(dist, ms_total / 1e3)
    value = reduce_sum(dist, args.steps) / t_max if world > 1 else args.steps / (ms_total / 1e3)

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
    e2e_el = reduce_max(dist, time.perf_counter() - t0)
    e2e = reduce_sum(dist, args.steps) / e2e_el

    peak, peak_kind = load_peaks()
    achieved = (alg_bytes / args.steps) / (ms_solver / args.steps / 1e3) / 1e9 if ms_solver > 0 else 0.0
    line = {
        "metric": "time steps/s at Stokes residual 1e-8", "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded .input, Philox initial temperature)",
        "config": {"workload": args.workload, "desc": wl["desc"], "mesh": wl["mesh"],
                   "parallelism": f"replicas x{world}", "l2": "flushed (256 MB write) between steps",
                   "uzawa_cycles_per_step": uz / args.steps, "cg_cycles_per_step": cgc / args.steps,
                   "max_stokes_residual": res},
        "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": 8 * nno,
                "d2h_bytes_per_step": 8 * (3 * nno + nel)},
        "gpu_launches": launches,
        "roofline": {"kernel": "k_uzawa (persistent Stokes solver)", "bound": "hbm", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": None, "alg_bytes_per_launch": alg_bytes / args.steps,
                     "ms_per_launch": ms_solver / args.steps},
        "clocks": clocks,
        "wall_s_timed": wall,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, el = cpu_sample(wl["input"], args.cpu_steps)
        line["cpu_baseline"] = {"value": v, "unit": "steps/s", "cores": 1, "kind": "port",
                                "sample": f"{args.cpu_steps} steady steps of {args.workload} ({el:.1f} s)"}
    model.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_gpu(args, wl)


if __name__ == "__main__":
    sys.exit(main())
