"""Build recipe for the reference programs used as checkers -- TEST
INFRASTRUCTURE ONLY.

Compiles the reference's box-source generator ``ntde_line`` from its own
sources where they lie (``PSV/psv_clean_double/source/source_line.cpp``,
``source/waveform.cpp``, ``param/param.cpp`` and ``getpar/getpar.cpp``, the
last as C) with ``g++``/``gcc`` directly, plus ``oracle/ref_convolve.cpp``
(a CPU restatement of the one CUDA kernel the program calls), into
``oracle/_ref/ntde_line``.  Only ``tests/golden/make_line_source.py`` and the
reference-pin tests run it; nothing ships with the product.  Without the
reference sources (e.g. on a machine that only has this repository) the
build is skipped and returns None.

``getpar.cpp`` compiles only as C, so ``oracle/ref_getpar_c.h`` is
force-included into ``param.cpp`` to give its getpar entry points C linkage.
``-ffp-contract=off`` keeps the compiler from fusing the reference's
products and sums on machines with FMA instructions, so the program's
arithmetic is the same on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
# The read-only reference checkout this recipe compiles from (the one place
# the repository names it); FD23_REFERENCE_ROOT points elsewhere.
REF_ROOT = os.environ.get("FD23_REFERENCE_ROOT") or "/root/reference"
PD = os.path.join(REF_ROOT, "PSV", "psv_clean_double")
NTDE = os.path.join(OUT_DIR, "ntde_line")


def sources():
    return {
        "source_line": os.path.join(PD, "source", "source_line.cpp"),
        "waveform": os.path.join(PD, "source", "waveform.cpp"),
        "param": os.path.join(PD, "param", "param.cpp"),
        "getpar": os.path.join(PD, "getpar", "getpar.cpp"),
        "convolve": os.path.join(HERE, "ref_convolve.cpp"),
        "getpar_c": os.path.join(HERE, "ref_getpar_c.h"),
    }


def build(force=False):
    src = sources()
    if not all(os.path.exists(p) for p in src.values()):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(NTDE):
        m = os.path.getmtime(NTDE)
        if all(os.path.getmtime(p) <= m for p in src.values()):
            return NTDE
    flags = ["-O2", "-w", "-ffp-contract=off"]
    objs = []
    for name, path in src.items():
        if path.endswith(".h"):
            continue
        obj = os.path.join(OUT_DIR, name + ".o")
        cc = ["gcc", "-x", "c"] if name == "getpar" else ["g++"]
        extra = ["-include", os.path.join(HERE, "ref_getpar_c.h")] if name == "param" else []
        subprocess.check_call(cc + flags + extra + ["-c", path, "-o", obj])
        objs.append(obj)
    subprocess.check_call(["g++", "-o", NTDE] + objs + ["-lm"])
    return NTDE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
