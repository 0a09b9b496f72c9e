"""Extract the reference's own known-answer data into small committed fixtures.

Run in a checkout where the fd23 reference tree is available::

    python tests/golden/make_golden.py /path/to/fd23

Reads only data files of the reference (seismograms, restart states, station
lists, model files) and writes:

  psv_fp64_golden.npz   PSV/psv_clean_double/test/0_U, 0_W (FP64, 2001 x 36)
                        with its station list and .mdl text
  psv_fp32_restart.npz  PSV/clean_nobox/TEST/tt/state000000, state000001,
                        state000499, state000999 (FP32 96x96 restart states)
  isis_headers.npz      the trace headers (bytes) of PSV/psv_clean_double/test/
                        0_U.isis, 0_W.isis (36 x 136-byte FP64 headers) and of
                        PSV/t/clean_nobox/TEST/output_U.isis (400 x 84-byte
                        FP32 headers); the traces themselves are the
                        seismograms above

The parameters of each run are stored next to the data.  Two of them differ
from the parfiles committed in the reference and were recovered from the data
themselves:
  * the restart states come from the top-absorbing build (psi arrays of the
    top PML are non-zero after one step) with vp = 6.8 (the fixtures' stress
    fields after two steps are reproduced only with vp = 6.8, not with the
    8.0 of the committed homo.mdl);
  * the FP64 golden matches its parfile exactly.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    pd = os.path.join(ref, "PSV", "psv_clean_double", "test")
    gu = np.fromfile(os.path.join(pd, "0_U"), dtype=np.float64).reshape(2001, 36)
    gw = np.fromfile(os.path.join(pd, "0_W"), dtype=np.float64).reshape(2001, 36)
    stations = np.array([int(t) for t in open(os.path.join(pd, "station200")).read().split()],
                        dtype=np.int32).reshape(-1, 2)  # (z, x) pairs
    mdl = open(os.path.join(pd, "homo.mdl")).read()
    np.savez_compressed(
        os.path.join(HERE, "psv_fp64_golden.npz"), seis_u=gu, seis_w=gw, stations_zx=stations,
        mdl=np.array(mdl),
        params=np.array(json.dumps(dict(nx=2048, nz=1024, h=0.3, dt=0.01, nt=2001, xs=1024, zs=100,
                             strike=0.0, dip=20.0, rake=90.0, azimuth=45.0, alpha=-5, stype=3,
                             npml=32, pml_r=1e-11, pml_dt=0.005, pml_v=30.0, pml_fc=2.0,
                             topabsorb=0, itrecord=1))))
    hdr = {}
    for c in ("U", "W"):
        raw = open(os.path.join(pd, "0_%s.isis" % c), "rb").read()
        step = 136 + 8 * 2001
        hdr["fp64_" + c] = np.frombuffer(raw, dtype=np.uint8).reshape(36, step)[:, :136].copy()
    raw = open(os.path.join(ref, "PSV", "t", "clean_nobox", "TEST", "output_U.isis"), "rb").read()
    step = 84 + 4 * 2000
    hdr["fp32_U"] = np.frombuffer(raw, dtype=np.uint8).reshape(400, step)[:, :84].copy()
    np.savez_compressed(os.path.join(HERE, "isis_headers.npz"), **hdr)
    tt = os.path.join(ref, "PSV", "clean_nobox", "TEST", "tt")
    states = {}
    for i in (0, 1, 499, 999):
        states["state%06d" % i] = np.fromfile(os.path.join(tt, "state%06d" % i), dtype=np.float32)
    np.savez_compressed(
        os.path.join(HERE, "psv_fp32_restart.npz"), **states,
        params=np.array(json.dumps(dict(nx=96, nz=96, h=0.3, dt=0.01, xs=33, zs=33, strike=0.0, dip=20.0,
                             rake=90.0, azimuth=45.0, alpha=-30, stype=3, npml=32, pml_r=1e-11,
                             pml_dt=0.005, pml_v=30.0, pml_fc=2.0, topabsorb=1, vp=6.8, vs=4.0,
                             den=3.0, station_zx=(0, 0)))))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FD23_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py /path/to/fd23 (or set FD23_REFERENCE_ROOT)")
    main(root)
