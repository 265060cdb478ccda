"""Build recipe for the oracle's C restatement (test infrastructure).

Compiles oracle/ref_cpu.c into oracle/_build/libsphref.so with gcc.  FMA
contraction is disabled so that FP64 results are the same on x86-64 and
aarch64 and follow the reference's operation order.

The reference (iwoplaza/cuda-sph) is Python with numba-CUDA kernels and has no
C/C++ sources, so there is no oracle/_ref build of the reference itself.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsphref.so")
SRC = os.path.join(HERE, "ref_cpu.c")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)
            and os.path.getmtime(LIB) >= os.path.getmtime(
                os.path.join(HERE, "..", "include", "sphgb.h"))):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
