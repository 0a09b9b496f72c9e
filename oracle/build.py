"""Build recipe for the fd23 CPU oracle (test infrastructure only).

Compiles ``oracle/fd23_oracle.c`` into ``oracle/_build/libfd23_oracle.so``.
The oracle is the checker used by ``tests/``, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``; the product library never loads it.

``-ffp-contract=off`` keeps the compiler from fusing multiply-adds on its own:
every fused multiply-add in the oracle is an explicit ``fma()`` call, which is
what lets the oracle and the CUDA kernels agree bit for bit.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfd23_oracle.so")
SRCS = [os.path.join(HERE, "fd23_oracle.c"), os.path.join(HERE, "fd23_oracle_step.inc")]


def _flags():
    flags = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11"]
    # hardware FMA so fma() is one instruction; results are the same
    # correctly-rounded values as the libm fallback on any machine
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")
    return flags


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        lib_m = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= lib_m for s in SRCS):
            return LIB
    cmd = ["gcc"] + _flags() + ["-o", LIB, SRCS[0], "-lm"]
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
