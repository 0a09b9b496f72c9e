"""Build the fd23 engine library in-tree: fd23_gb300/_lib/libfd23.so.

Compiles every translation unit under fd23_gb300/csrc/ for sm_103a with nvcc
(host C++ through nvcc as well, so the CUDA headers are on the path), in
parallel, and links one shared library exporting the C ABI of include/fd23.h.

-fmad=false: no implicit multiply-add contraction; every fused multiply-add
in the kernels is written out, which makes results bitwise reproducible.
-ffp-contract=off does the same for the host set-up code.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libfd23.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "fd23.h"))
    return hs


def _compile(src, verbose=False):
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    cmd = [_nvcc(), "-c", src, "-o", obj, "-std=c++17", "-O3", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-O2"]
    if src.endswith(".cu"):
        cmd += ARCH + ["-lineinfo", "-fmad=false"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd += ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


CLI_SRC = os.path.join(HERE, "cli", "fd23_psv2d.cpp")
CLI = os.path.join(LIBDIR, "fd23_psv2d")
CLI_SH = os.path.join(LIBDIR, "fd23_sh2d")
CLI_NTDE = os.path.join(LIBDIR, "fd23_ntde_line")


def build_cli(force=False):
    """The parfile programs fd23_psv2d, fd23_sh2d and fd23_ntde_line (one
    source) next to the library, linked to it and finding it through their
    own directory."""
    newest = max(os.path.getmtime(p) for p in [CLI_SRC, LIB] + headers())
    for exe, flag in ((CLI, "-DFD23_CLI_SH=0"), (CLI_SH, "-DFD23_CLI_SH=1"), (CLI_NTDE, "-DFD23_CLI_NTDE=1")):
        if not force and os.path.exists(exe) and os.path.getmtime(exe) >= newest:
            continue
        cmd = [_nvcc(), "-x", "c++", "-std=c++17", "-O2", flag, CLI_SRC, "-o", exe,
               "-L" + LIBDIR, "-lfd23", "-Xlinker", "-rpath=$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("cli build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return CLI


def build(force=False, verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = sources()
    newest = max(os.path.getmtime(p) for p in srcs + headers() + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        build_cli(force)
        return LIB
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    objs = [o for o, _ in results]
    cmd = [_nvcc(), "-shared", "-o", LIB] + objs + ARCH
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    build_cli(True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
