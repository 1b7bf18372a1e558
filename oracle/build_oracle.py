"""Build the CPU oracle (test infrastructure): oracle/liboracle.so from oracle.c.

Compiled with -ffp-contract=off so that x86 and Arm hosts evaluate every
expression with the same roundings, and with OpenMP when the compiler has it
(the CPU baseline may use all host cores; one thread keeps the reference's
summation order).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.c")
# the seeded initial-temperature header shared with the engine and the dump harness
IC_DIR = os.path.join(os.path.dirname(HERE), "mantle_convection_lab_gb300", "csrc", "host")
LIB = os.path.join(HERE, "liboracle.so")


def build():
    deps = [SRC, os.path.join(IC_DIR, "mclg_ic.h")]
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) > os.path.getmtime(d) for d in deps):
        return LIB
    # built beside the library and renamed over it, so that a process that has
    # the old one loaded keeps a consistent file
    tmp = LIB + f".{os.getpid()}.tmp"
    base = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-I" + IC_DIR, SRC, "-o", tmp,
            "-lm"]
    p = subprocess.run(base[:1] + ["-fopenmp"] + base[1:], capture_output=True, text=True)
    if p.returncode != 0:
        p = subprocess.run(base, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + p.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build())
