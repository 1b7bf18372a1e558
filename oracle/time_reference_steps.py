"""Time whole steps of the reference's algorithm (the CPU oracle) on an input --
test and measurement infrastructure, never part of the product.

    python oracle/time_reference_steps.py <file.input> <steps> [threads] > out.json

Runs `steps` whole time steps (buoyancy .. Uzawa solve .. temperature update,
with the reference's own stopping rules and caps) from the input's initial
temperature on a uniform mesh, with the oracle's standalone mesh (nothing of
the engine is loaded), and prints one JSON object: per step the wall time,
Uzawa cycles, inner CG iterations and the true Stokes residuals.
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import oracle_port  # noqa: E402


def main():
    path, steps = sys.argv[1], int(sys.argv[2])
    threads = int(sys.argv[3]) if len(sys.argv) > 3 else (os.cpu_count() or 1)
    t0 = time.perf_counter()
    o = oracle_port.Oracle(path, threads=threads, standalone=True)
    setup = time.perf_counter() - t0
    out = {"input": os.path.basename(path), "threads": threads, "setup_s": setup, "nno": o.nno, "nel": o.nel,
           "steps": []}
    for s in range(steps):
        t0 = time.perf_counter()
        st = o.step()
        el = time.perf_counter() - t0
        out["steps"].append({"step": s, "wall_s": el, "uzawa_cycles": st["uzawa_cycles"],
                             "cg_iterations": st["cg_cycles"], "heat_cg_iterations": st["heat_cg_cycles"],
                             "res_momentum": float(st["res_m"]), "res_continuity": float(st["res_c"])})
        print(json.dumps(out["steps"][-1]), file=sys.stderr, flush=True)
    o.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
