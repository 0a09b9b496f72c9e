"""Build recipe for the reference programs used as checkers -- TEST
INFRASTRUCTURE ONLY.

Two kinds of checker are built, both from the reference's own sources:

* ``oracle/_ref/ntde_line``, the box-source generator (below);
* ``oracle/_ref/ref_setup_pn``, ``ref_setup_sh``, ``ref_setup_pd``: the
  harness ``oracle/ref_setup_harness.cpp`` linked with the host set-up code
  of the FP32 P-SV program (``PSV/clean_nobox``: material, cpml, model), the
  SH program (``SH``: the same plus ``fd/fd.cpp``'s host step) and the FP64
  P-SV program (``PSV/psv_clean_double``: the same plus ``box/box.cpp``,
  ``field/field.cpp`` and ``fd/fd.cpp``'s residual updates).  Only
  ``tests/golden/make_ref_pins.py`` runs them.

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


# harness programs: name -> (program root, -D macro, program sources)
HARNESS = {
    "ref_setup_pn": (os.path.join("PSV", "clean_nobox"), "REF_PN",
                     ["material/material.cpp", "cpml/cpml.cpp", "model/model.cpp", "model/util.cpp"]),
    "ref_setup_sh": ("SH", "REF_SH",
                     ["material/material.cpp", "cpml/cpml.cpp", "model/model.cpp", "model/util.cpp",
                      "fd/fd.cpp"]),
    "ref_setup_pd": (os.path.join("PSV", "psv_clean_double"), "REF_PD",
                     ["material/material.cpp", "cpml/cpml.cpp", "model/model.cpp", "model/util.cpp",
                      "fd/fd.cpp", "box/box.cpp", "field/field.cpp"]),
}


def build_harness(force=False):
    """The three set-up harnesses; {name: path}, or None without the
    reference sources."""
    harness = os.path.join(HERE, "ref_setup_harness.cpp")
    out = {}
    for name, (sub, macro, files) in HARNESS.items():
        root = os.path.join(REF_ROOT, sub)
        srcs = [os.path.join(root, f) for f in files]
        if not all(os.path.exists(p) for p in srcs):
            return None
        os.makedirs(OUT_DIR, exist_ok=True)
        exe = os.path.join(OUT_DIR, name)
        if force or not os.path.exists(exe) or any(
                os.path.getmtime(p) > os.path.getmtime(exe) for p in srcs + [harness]):
            subprocess.check_call(["g++", "-std=c++11", "-O2", "-w", "-ffp-contract=off", "-D" + macro,
                                   "-I" + root, "-o", exe, harness] + srcs + ["-lm"])
        out[name] = exe
    return out


def build(force=False):
    build_harness(force)
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
