"""Golden vectors of the reference's box-source generator.

Run in a checkout where the fd23 reference tree is available::

    python tests/golden/make_line_source.py [/path/to/fd23]

Builds the reference program ``ntde_line`` from its own sources with
``oracle/build_ref.py`` (its one CUDA kernel, the wavelet convolution, is
restated for the CPU in ``oracle/ref_convolve.cpp``), runs it on the parfiles
below in a temporary directory and writes ``line_source_ref.npz``: for each
case its parameters, every 10th frame of the U and W planes (at most 20), every frame of
a few cells, and the NaN mask of the whole output (cells within one step's
travel of the source divide 0 by 0 at t = 0).
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# name: (bw, nt, h, dt, vp, vs, den, source-time line, strike dip rake azimuth)
CASES = {
    "gauss_bw8": (8, 100, 5.0, 4e-4, 3000.0, 1730.0, 2500.0, "sourcetime=gaussian alpha=-8", (30, 60, 90, 0)),
    "trap_bw9": (9, 300, 5.0, 4e-4, 3000.0, 1730.0, 2500.0,
                 "sourcetime=trapezoid trap1=0.004 trap2=0.008 trap3=0.006", (10, 45, 30, 75)),
    "nan_bw12": (12, 200, 1.0, 4e-4, 3000.0, 1730.0, 2500.0, "sourcetime=gaussian alpha=5", (0, 90, 0, 20)),
    "long_bw16": (16, 2000, 10.0, 1e-3, 4000.0, 2300.0, 2.6, "sourcetime=gaussian alpha=-20", (200, 35, -60, 110)),
}
CELLS = ((0, 0), (3, 5), (7, 2), (5, 7))  # (plane x, plane z) of the full-length series, scaled by bw below


def stride(nt):
    """Frame stride of the stored planes: every 10th frame, at most 20 frames."""
    return max(10, nt // 20)


def parfile(name, bw, nt, h, dt, vp, vs, den, stf, mech):
    return (f"usebox=1 usepunch=0 ngpu=1\nnx=256 nz=256 nt={nt} h={h} dt={dt}\n"
            f"srcden={den} srcsvel={vs} srcpvel={vp} sourcefile=planes_{name}.bin bw={bw}\n{stf}\n"
            f"strike={mech[0]} dip={mech[1]} rake={mech[2]} azimuth={mech[3]}\n"
            f"xs=128 zs=128 npml=20 pml_dt={dt} pml_v=600 pml_r=1e-11 pml_fc=15\n"
            "itrecord=1 output=out nrec=1 ixrec0=10 izrec0_u=0 izrec0_w=0 idxrec=1 idzrec=0\n"
            "model=none.mdl ntsnap=100000\n")


def main(ref_root=None):
    if ref_root:
        os.environ["FD23_REFERENCE_ROOT"] = ref_root
    sys.path.insert(0, ROOT)
    from oracle import build_ref
    exe = build_ref.build()
    if exe is None:
        raise SystemExit("reference sources not found")
    out = {}
    meta = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (bw, nt, h, dt, vp, vs, den, stf, mech) in CASES.items():
            with open(os.path.join(tmp, name + ".par"), "w") as f:
                f.write(parfile(name, bw, nt, h, dt, vp, vs, den, stf, mech))
            subprocess.check_call([exe, f"par={name}.par"], cwd=tmp, stdout=subprocess.DEVNULL)
            n = bw + 8
            pl = np.fromfile(os.path.join(tmp, f"planes_{name}.bin"), dtype=np.float64).reshape(nt, 2, n, n)
            cells = np.array([(min(n - 1, cx * n // 8), min(n - 1, cz * n // 8)) for cx, cz in CELLS], np.int32)
            out[name + "_frames"] = pl[::stride(nt)]
            out[name + "_cells"] = cells
            out[name + "_series"] = np.stack([pl[:, :, cz, cx] for cx, cz in cells])  # [cell, t, comp]
            out[name + "_nan"] = np.packbits(np.isnan(pl).ravel())
            meta[name] = dict(bw=bw, nt=nt, h=h, dt=dt, vp=vp, vs=vs, den=den, stf=stf, mech=list(mech))
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "line_source_ref.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
