"""In-tree build of the engine library and its command-line driver.

    python -m mantle_convection_lab_gb300._build     (or __graft_entry__.build())

Produces
    mantle_convection_lab_gb300/libmclg.so   C ABI of include/mclg.h (host C + CUDA sm_103a)
    mantle_convection_lab_gb300/mclg_run     the Main.c-style driver: mclg_run <file.input>
Objects go to mantle_convection_lab_gb300/_build/.  Translation units compile
in parallel; only stale ones are rebuilt.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libmclg.so")
RUN = os.path.join(PKG, "mclg_run")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"] + ARCH
CC_FLAGS = ["-O2", "-std=gnu11", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra", "-Wno-unused-parameter"]

HOST_SRCS = ["host/mclg_input.c", "host/mclg_mesh.c", "host/mclg_output.c", "host/mclg_mesh_api.c", "host/mclg_amr.c", "host/mclg_refmg.c", "host/mclg_qtmg.c", "host/mclg_grain.c"]
CUDA_SRCS = ["cuda/k_elem.cu", "cuda/k_uzawa.cu", "cuda/k_heat.cu", "cuda/k_mg.cu", "cuda/k_cnn.cu", "cuda/k_amr.cu", "cuda/k_qt.cu", "cuda/k_mesh.cu", "cuda/mclg_writer.cu", "cuda/mclg_ctx.cu"]
HEADERS = ["host/mclg_host.h", "host/mclg_ic.h", "cuda/mclg_dev.cuh", "cuda/cg_solve.cuh", "cuda/k_mg.cuh", "cuda/k_tile.cuh", "cuda/cnn.cuh", "cuda/mclg_writer.cuh", "cuda/k_qt.cuh", "cuda/team.cuh"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd, log):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    if log is not None:
        log.append((" ".join(cmd), p.stdout + p.stderr))


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "mclg.h")]
    jobs, objs, log = [], [], []
    for src in HOST_SRCS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append(["gcc"] + CC_FLAGS + ["-I" + INCLUDE, "-c", s, "-o", o])
    for src in CUDA_SRCS:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([nvcc()] + NVCC_FLAGS + ["-I" + INCLUDE, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        list(ex.map(lambda c: _run(c, log), jobs))
    if jobs or not os.path.exists(LIB):
        _run([nvcc(), "-shared"] + ARCH + ["-o", LIB] + objs + ["-lpthread", "-ldl", "-lrt", "-lm"], log)
    drv = os.path.join(CSRC, "host", "mclg_run.c")
    if os.path.exists(drv) and (_stale(RUN, [drv, LIB])):
        _run(["gcc"] + CC_FLAGS + ["-I" + INCLUDE, drv, "-o", RUN, "-L" + PKG, "-lmclg",
              "-Wl,-rpath,$ORIGIN", "-lm"], log)
    if verbose:
        for cmd, out in log:
            print(cmd)
            if out.strip():
                print(out)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
