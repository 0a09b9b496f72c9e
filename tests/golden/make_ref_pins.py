"""Run the reference programs' own host code (built from its sources by
oracle/build_ref.py, oracle/ref_setup_harness.cpp) on seeded inputs and
store inputs and outputs as the fixture tests/golden/ref_pins.npz, which
tests/test_ref_pins_cpu.py compares the oracle against.

Run where the fd23 reference tree is available::

    python tests/golden/make_ref_pins.py /path/to/fd23

What is pinned (reference files relative to the fd23 project root):

  pn_*   PSV/clean_nobox (FP32 P-SV): MATERIAL::get_model
         (material/material.cpp) and CPML::CPML (cpml/cpml.cpp) on the 96 x 96
         homogeneous model of the FP32 restart states and on a seeded layered
         model with a fluid layer.
  sh_*   SH: MATERIAL::get_model (material/material.cpp:68-172: BV, the
         harmonic means MUX, MUZ with their row wrap), CPML::CPML
         (cpml/cpml.cpp:172-176 offsets), and one host step (fd/fd.cpp:43,121
         step_stress, step_velocity) from a seeded state.
  pd*_*  PSV/psv_clean_double (FP64 P-SV): MATERIAL::get_model, CPML::CPML,
         BOX::init_box (box/box.cpp:10-118 ring lists; the box material of
         MATERIAL::init_for_box_from_full, material/material.cpp:39-97),
         BOX::setboxsource (box.cpp:120-196) over the frames of a seeded
         displacement-plane file, and the residual updates step_stress_r /
         step_velocity_r (fd/fd.cpp:63,208) from a seeded residual field; two
         boxes, widths 20 and 17.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

PML = dict(pml_dt=0.005, pml_r=1e-11, pml_v=30.0, pml_fc=2.0)


def layered(nx, nz, seed, fluid=None):
    """seeded flat layers with a smooth lateral perturbation (km/s, g/cc)"""
    rng = np.random.default_rng(seed)
    bounds = np.sort(rng.integers(nz // 8, nz - 2, size=3))
    vel = rng.uniform(3.0, 6.0, size=4)
    layer = np.searchsorted(bounds, np.arange(nz), side="right")
    vp = np.repeat(vel[layer][:, None], nx, axis=1)
    vp *= 1.0 + 0.04 * np.sin(np.linspace(0, 5, nx))[None, :] * np.cos(np.linspace(0, 3, nz))[:, None]
    vs = vp / 1.73
    den = 0.31 * vp ** 0.25 * 8.0
    if fluid is not None:
        vs[fluid[0]:fluid[1], :] = 0.0
    return vp.astype(np.float32), vs.astype(np.float32), den.astype(np.float32)


def write_rasters(d, vp, vs, den):
    prefix = os.path.join(d, "m")
    for ext, a in (("vp", vp), ("vs", vs), ("den", den)):
        np.ascontiguousarray(a, dtype=np.float32).tofile(prefix + "." + ext)
    return prefix


def run(exe, args):
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s failed (%d): %s %s" % (exe, r.returncode, r.stdout, r.stderr))


def main(ref):
    sys.path.insert(0, ROOT)
    os.environ["FD23_REFERENCE_ROOT"] = ref
    from oracle import build_ref
    exes = build_ref.build_harness(force=True)
    if exes is None:
        sys.exit("reference sources not found under %s" % ref)
    fx = {}
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "out.bin")
        # ---- FP32 P-SV set-up ----
        cases = {"pn_restart": (96, 96, 0.3, 0.01, 32, (np.full((96, 96), 6.8, np.float32),
                                                         np.full((96, 96), 4.0, np.float32),
                                                         np.full((96, 96), 3.0, np.float32))),
                 "pn_layered": (72, 56, 0.3, 0.01, 10, layered(72, 56, 31, fluid=(20, 26)))}
        for key, (nx, nz, h, dt, npml, model) in cases.items():
            prefix = write_rasters(d, *model)
            run(exes["ref_setup_pn"], [nx, nz, h, dt, npml, PML["pml_dt"], PML["pml_r"], PML["pml_v"],
                                       PML["pml_fc"], prefix, out])
            raw = np.fromfile(out, np.float32)
            n = nx * nz
            fx[key + "_in"] = np.stack(model)
            fx[key + "_geom"] = np.array([nx, nz, npml], np.int32)
            fx[key + "_hdt"] = np.array([h, dt])
            fx[key + "_mat"] = raw[:5 * n].reshape(5, nz, nx)
            fx[key + "_bck"] = raw[5 * n:]
        # ---- SH set-up and one host step ----
        nx, nz, h, dt, npml = 72, 56, 0.3, 0.01, 10
        model = layered(nx, nz, 37)
        prefix = write_rasters(d, *model)
        rng = np.random.default_rng(41)
        state = rng.standard_normal((3, nz, nx)).astype(np.float32)
        sfile = os.path.join(d, "state.bin")
        state.tofile(sfile)
        run(exes["ref_setup_sh"], [nx, nz, h, dt, npml, PML["pml_dt"], PML["pml_r"], PML["pml_v"],
                                   PML["pml_fc"], prefix, out, sfile])
        raw = np.fromfile(out, np.float32)
        n = nx * nz
        fx["sh_in"] = np.stack(model)
        fx["sh_geom"] = np.array([nx, nz, npml], np.int32)
        fx["sh_hdt"] = np.array([h, dt])
        fx["sh_mat"] = raw[:3 * n].reshape(3, nz, nx)
        nb = 3 * 2 * (nx + nz)
        fx["sh_bck"] = raw[3 * n:3 * n + nb]
        fx["sh_state_in"] = state
        fx["sh_state_out"] = raw[3 * n + nb:].reshape(3, nz, nx)
        # ---- FP64 P-SV set-up, box, residual step ----
        for key, (nx, nz, npml, xs, zs, bw, seed) in {"pd20": (72, 64, 10, 36, 32, 20, 43),
                                                       "pd17": (72, 64, 10, 33, 30, 17, 47)}.items():
            h, dt = 0.3, 0.01
            model = layered(nx, nz, seed, fluid=(50, 54))
            src = (6.0, 3.4, 2.7)  # srcpvel srcsvel srcden
            if key == "pd17":
                # the upper half of the box (and its neighbours) already in the
                # source material: those cells keep theirs, the others are replaced
                x0, z0 = xs + (bw + 1) // 2 + 1 - bw, zs + (bw + 1) // 2 + 1 - bw
                for a, v in zip(model, src):
                    a[z0 - 1:z0 + bw // 2, x0 - 1:x0 + bw + 1] = v
            prefix = write_rasters(d, *model)
            frames = 4
            rng = np.random.default_rng(seed + 1)
            planes = rng.standard_normal((frames, 2, bw + 8, bw + 8)) * 1e-3
            pfile = os.path.join(d, "planes.bin")
            planes.tofile(pfile)
            resid = rng.standard_normal((5, bw, bw))
            rfile = os.path.join(d, "resid.bin")
            resid.tofile(rfile)
            run(exes["ref_setup_pd"], [nx, nz, h, dt, npml, PML["pml_dt"], PML["pml_r"], PML["pml_v"],
                                       PML["pml_fc"], prefix, out, xs, zs, bw, src[0], src[1], src[2], pfile,
                                       frames, rfile])
            raw = open(out, "rb").read()
            n = nx * nz
            o = 0

            def take(count, dtype):
                nonlocal o
                a = np.frombuffer(raw, dtype=dtype, count=count, offset=o)
                o += count * np.dtype(dtype).itemsize
                return a.copy()

            fx[key + "_in"] = np.stack(model)
            fx[key + "_geom"] = np.array([nx, nz, npml, xs, zs, bw], np.int32)
            fx[key + "_hdt_src"] = np.array([h, dt, *src])
            fx[key + "_mat"] = take(5 * n, np.float64).reshape(5, nz, nx)
            fx[key + "_bck"] = take(3 * 4 * (nx + nz), np.float64)
            head = take(4, np.int32)
            nsub, nadd = int(head[0]), int(head[1])
            fx[key + "_box_head"] = head
            fx[key + "_r_sub"] = take(nsub, np.int32)
            fx[key + "_a_sub"] = take(nsub, np.int32)
            fx[key + "_r_add"] = take(nadd, np.int32)
            fx[key + "_a_add"] = take(nadd, np.int32)
            fx[key + "_bmat"] = take(5 * bw * bw, np.float64).reshape(5, bw, bw)
            fx[key + "_planes"] = planes
            fx[key + "_sfield"] = take((frames - 1) * 5 * bw * bw, np.float64).reshape(frames - 1, 5, bw, bw)
            fx[key + "_resid_in"] = resid
            fx[key + "_resid_out"] = take(5 * bw * bw, np.float64).reshape(5, bw, bw)
            assert o == len(raw)
    np.savez_compressed(os.path.join(HERE, "ref_pins.npz"), **fx)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FD23_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_ref_pins.py /path/to/fd23 (or set FD23_REFERENCE_ROOT)")
    main(root)
