"""GPU parity: the CUDA product (through the C ABI) against the CPU oracle.

FP32 and FP64 are bit-exact (same inputs, same canonical operation order),
for the fused single-pass sweep and for the two-pass sweep, over grid sizes
that are not multiples of the tile sizes, free-surface and absorbing tops,
every point-source kind, the fluid-layer edge rules and record decimation.
The reduced-storage forms (BF16, FP16) are checked against the FP64 oracle
with the tolerance stated in each test.
"""
import json
import os

import numpy as np
import pytest

from oracle import fd23_oracle as O
from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _run(case, prec, kernel, nt=None, itrecord=1):
    s = case.solver(prec, kernel)
    s.run(case.nt if nt is None else nt, itrecord)
    out = [s.seismograms(0)] + ([s.seismograms(1)] if case.wave == "psv" else [])
    st = s.get_state()
    s.close()
    return out, st


PSV_CASES = [
    dict(nx=96, nz=64, kind=3),
    dict(nx=250, nz=130, kind=3, topabsorb=1),
    dict(nx=257, nz=131, kind=13, npml=16),
    dict(nx=300, nz=200, kind=1, fluid=True),
    dict(nx=130, nz=97, kind=3, zs=1, xs=5),           # source next to the surface and edge
]


@pytest.mark.parametrize("kernel", ["fused", "twopass"])
@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("cfg", PSV_CASES, ids=lambda c: "%dx%d_k%d" % (c["nx"], c["nz"], c["kind"]))
def test_psv_bit_exact(cfg, prec, kernel):
    case = Case("psv", nt=70, **cfg)
    ref, ref_state = case.oracle(prec)
    got, state = _run(case, prec, kernel)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)
    np.testing.assert_array_equal(state, ref_state)


SH_CASES = [
    dict(nx=96, nz=64, kind=3),
    dict(nx=250, nz=130, kind=2, topabsorb=1),
    dict(nx=257, nz=131, kind=13, npml=16),
    dict(nx=140, nz=90, kind=2, zs=0, xs=3),
]


@pytest.mark.parametrize("kernel", ["fused", "twopass"])
@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("cfg", SH_CASES, ids=lambda c: "%dx%d_k%d" % (c["nx"], c["nz"], c["kind"]))
def test_sh_bit_exact(cfg, prec, kernel):
    case = Case("sh", nt=70, **cfg)
    ref, ref_state = case.oracle(prec)
    got, state = _run(case, prec, kernel)
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(state, ref_state)


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_multi_item_worklist_bit_exact(wave):
    """1000x1000: CTAs own pieces of two strips (item boundaries inside a CTA)."""
    case = Case(wave, 1000, 1000, npml=20, nt=40, seed=3)
    ref, ref_state = case.oracle("f32")
    got, state = _run(case, "f32", "fused")
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)
    np.testing.assert_array_equal(state, ref_state)


def test_itrecord_and_split_runs():
    """records every 3rd step; 0..N in several run() calls equals one call."""
    case = Case("psv", 200, 120, nt=50, seed=5)
    ref, _ = case.oracle("f32", itrecord=3)
    s = case.solver("f32", "fused")
    s.run(17, 3)
    s.run(20, 3)
    s.run(13, 3)
    np.testing.assert_array_equal(s.seismograms(0), ref[0])
    np.testing.assert_array_equal(s.seismograms(1), ref[1])
    assert s.step == 50
    s.close()


def test_state_roundtrip_restart():
    """get_state after k steps, set_state into a fresh solver, continue:
    identical to an uninterrupted run (PN savestate / restart path)."""
    case = Case("psv", 180, 140, nt=60, seed=7, topabsorb=1)
    _, full_state = case.oracle("f32", nt=60)
    a = case.solver("f32")
    a.run(25)
    st = a.get_state()
    a.close()
    b = case.solver("f32")
    b.set_state(st, 25)
    b.run(35)
    np.testing.assert_array_equal(b.get_state(), full_state)
    b.close()


def test_fp64_golden_on_gpu():
    """PSV/psv_clean_double/test/0_U, 0_W through the product, FP64 fused
    sweep: bit for bit, 2001 steps, 36 traces."""
    d = np.load(os.path.join(GOLD, "psv_fp64_golden.npz"))
    p = json.loads(str(d["params"]))
    import tempfile
    import fd23_gb300 as F
    with tempfile.NamedTemporaryFile("w", suffix=".mdl", delete=False) as fh:
        fh.write(str(d["mdl"]))
        mdl = fh.name
    nx, nz, h, dt = p["nx"], p["nz"], p["h"], p["dt"]
    vp, vs, den = O.mdl_raster(O.parse_mdl(mdl), nx, nz, h)
    os.unlink(mdl)
    s = F.Solver("psv", nx, nz, p["npml"], h, dt, prec="f64", pml_dt=p["pml_dt"],
                 pml_r=p["pml_r"], pml_v=p["pml_v"], pml_fc=p["pml_fc"])
    s.set_model(vp, vs, den)
    src = F.wavelet_gaussian(dt, p["alpha"])
    s.set_source(p["stype"], p["xs"], p["zs"], F.moment_psv(p["strike"], p["dip"], p["rake"],
                                                            p["azimuth"]), src, p["nt"])
    rx, rz = [], []
    for z, x in d["stations_zx"]:
        rx += [x, x - 1]
        rz += [z, z]
    s.set_receivers(0, rx, rz)
    s.set_receivers(1, rx, rz)
    s.run(p["nt"])
    np.testing.assert_array_equal(s.seismograms(0), d["seis_u"])
    np.testing.assert_array_equal(s.seismograms(1), d["seis_w"])
    s.close()


def test_fp32_restart_fixture_on_gpu():
    """PSV/clean_nobox/TEST/tt/state000499 -> 500 steps -> state000999."""
    d = np.load(os.path.join(GOLD, "psv_fp32_restart.npz"))
    p = json.loads(str(d["params"]))
    import fd23_gb300 as F
    nx, nz, h, dt = p["nx"], p["nz"], p["h"], p["dt"]
    s = F.Solver("psv", nx, nz, p["npml"], h, dt, prec="f32", topabsorb=p["topabsorb"],
                 pml_dt=p["pml_dt"], pml_r=p["pml_r"], pml_v=p["pml_v"], pml_fc=p["pml_fc"])
    s.set_model(np.full((nz, nx), p["vp"]), np.full((nz, nx), p["vs"]), np.full((nz, nx), p["den"]))
    s.set_source(p["stype"], p["xs"], p["zs"], F.moment_psv(p["strike"], p["dip"], p["rake"],
                                                            p["azimuth"]),
                 F.wavelet_gaussian(dt, p["alpha"]), 1000)
    s.set_state(d["state000499"], 500)
    s.run(500)
    got = s.get_state()
    n = nx * nz
    g = d["state000999"]
    errs = [O.rel_l2(got[k * n:(k + 1) * n], g[k * n:(k + 1) * n]) for k in range(5)]
    assert max(errs[2:]) < 1e-5, errs
    assert max(errs[:2]) < 1e-3, errs
    s.close()


@pytest.mark.parametrize("prec", ["bf16", "f16"])
@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_reduced_storage_fused_equals_twopass(prec, wave):
    """Both sweeps round through the same storage at the same points."""
    case = Case(wave, 257, 131, nt=60, seed=11)
    a, sa = _run(case, prec, "fused")
    b, sb = _run(case, prec, "twopass")
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(sa, sb)


# measured on GB300 (400 steps): P-SV BF16 4.3e-2 / 2.1e-2, FP16 2.9e-3 / 3.2e-3;
# SH BF16 3.1e-2, FP16 2.7e-3.  Rounding the material to 16 bits alone gives
# 1.2e-3 (FP16) and 3.4e-2 (BF16) on this case (FP32 oracle, rounded material).
RS_TOL = {("psv", "bf16"): 6e-2, ("psv", "f16"): 5e-3, ("sh", "bf16"): 5e-2, ("sh", "f16"): 5e-3}


@pytest.mark.parametrize("prec", ["bf16", "f16"])
@pytest.mark.parametrize("wave,kind", [("psv", 3), ("sh", 2)])
def test_reduced_storage_accuracy(wave, kind, prec):
    """Seismogram relative L2 of the 16-bit storage forms against the FP64
    oracle, 400 steps, receivers inside the wave's reach (tolerances in
    RS_TOL; FP32 on the same case is at ~1e-6)."""
    case = Case(wave, 240, 160, nt=400, seed=13, xs=120, zs=20, kind=kind, wavelet=("gauss", -8))
    ref, _ = case.oracle("f64")
    got, _ = _run(case, prec, "fused")
    errs = [O.rel_l2(g, r) for g, r in zip(got, ref)]
    print("reduced storage", wave, prec, errs)
    assert max(errs) < RS_TOL[(wave, prec)], errs


def test_norm2_watchdog():
    case = Case("psv", 128, 96, nt=30, seed=2)
    s = case.solver("f32")
    s.run(30)
    _, st = case.oracle("f32", nt=30)
    n = 128 * 96
    assert abs(s.norm2() - float(np.sum(st[:5 * n].astype(np.float64) ** 2))) < 1e-9 * max(1.0, s.norm2())
    s.close()
