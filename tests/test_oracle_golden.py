"""The CPU oracle against the reference's own known-answer data.

* PSV/psv_clean_double/test/0_U, 0_W: FP64 P-SV with a fluid layer,
  2048x1024, 2001 steps, dip-slip moment source, 18 stations.  The oracle
  reproduces it bit for bit.
* PSV/clean_nobox/TEST/tt/state*: FP32 P-SV restart states (96x96, top
  absorbing boundary).  The oracle reproduces them to FP32 round-off and the
  state layout round-trips through a restart.
"""
import json
import os

import numpy as np
import pytest

from oracle import fd23_oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _psv_setup_fp64(d, p, tmp_path):
    mdl = tmp_path / "homo.mdl"
    mdl.write_text(str(d["mdl"]))
    nx, nz, h, dt = p["nx"], p["nz"], p["h"], p["dt"]
    vp, vs, den = O.mdl_raster(O.parse_mdl(str(mdl)), nx, nz, h)
    mat, stab, rc = O.psv_material(vp, vs, den, h, dt)
    assert rc == 0 and stab < 1.0
    bck = O.cpml_psv(nx, nz, p["npml"], p["pml_dt"], p["pml_r"], p["pml_v"], p["pml_fc"])
    src = O.gaussian(dt, p["alpha"])
    m = O.moment_psv(p["strike"], p["dip"], p["rake"], p["azimuth"])
    terms = O.source_terms("psv", p["stype"], nx, p["xs"], p["zs"], m, h, dt, src, p["nt"])
    st = d["stations_zx"]
    rx, rz = [], []
    for z, x in st:
        rx += [x, x - 1]
        rz += [z, z]
    rec = np.array(rx) + np.array(rz) * nx
    return mat, bck, terms, rec


def test_fp64_golden_bit_exact(tmp_path):
    d = np.load(os.path.join(GOLD, "psv_fp64_golden.npz"))
    p = json.loads(str(d["params"]))
    mat, bck, terms, rec = _psv_setup_fp64(d, p, tmp_path)
    nt = p["nt"]
    su, sw, _ = O.psv_run("f64", p["nx"], p["nz"], p["npml"], p["topabsorb"], mat, bck, terms, rec,
                          rec, nt)
    np.testing.assert_array_equal(su, d["seis_u"][:nt])
    np.testing.assert_array_equal(sw, d["seis_w"][:nt])


def _restart_setup():
    d = np.load(os.path.join(GOLD, "psv_fp32_restart.npz"))
    p = json.loads(str(d["params"]))
    nx, nz, h, dt = p["nx"], p["nz"], p["h"], p["dt"]
    vp = np.full((nz, nx), p["vp"])
    vs = np.full((nz, nx), p["vs"])
    den = np.full((nz, nx), p["den"])
    mat, _, _ = O.psv_material(vp, vs, den, h, dt)
    bck = O.cpml_psv(nx, nz, p["npml"], p["pml_dt"], p["pml_r"], p["pml_v"], p["pml_fc"])
    src = O.gaussian(dt, p["alpha"])
    m = O.moment_psv(p["strike"], p["dip"], p["rake"], p["azimuth"])
    terms = O.source_terms("psv", p["stype"], nx, p["xs"], p["zs"], m, h, dt, src, 1000)
    z, x = p["station_zx"]
    rec = np.array([x + z * nx, x - 1 + z * nx])
    return d, p, mat, bck, terms, rec


def _field_errs(s, g, nx, nz):
    n = nx * nz
    return [O.rel_l2(s[k * n:(k + 1) * n], g[k * n:(k + 1) * n]) for k in range(5)] + [
        O.rel_l2(s[5 * n:], g[5 * n:])]


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_fp32_restart_states(prec):
    d, p, mat, bck, terms, rec = _restart_setup()
    nx, nz = p["nx"], p["nz"]
    for nt, key, tol in ((1, "state000000", 1e-6), (2, "state000001", 1e-6),
                         (500, "state000499", 5e-5)):
        _, _, s = O.psv_run(prec, nx, nz, p["npml"], p["topabsorb"], mat, bck, terms, rec, rec, nt)
        errs = _field_errs(s, d[key], nx, nz)
        assert max(errs) < tol, (key, errs)


def test_fp32_restart_continuity():
    """state000499 -> 500 more steps -> state000999 (PN/main.cpp restart path)."""
    d, p, mat, bck, terms, rec = _restart_setup()
    nx, nz = p["nx"], p["nz"]
    _, _, s = O.psv_run("f32", nx, nz, p["npml"], p["topabsorb"], mat, bck, terms, rec, rec, 500,
                        it0=500, state=d["state000499"])
    errs = _field_errs(s, d["state000999"], nx, nz)
    # stresses and memory variables carry the signal; the velocities have
    # decayed to ~1e-6 of their peak and sit at the FP32 noise floor
    assert max(errs[2:]) < 1e-5, errs
    assert max(errs[:2]) < 1e-3, errs


def test_restart_split_is_exact():
    """Running 0..N in one go equals 0..k then k..N through the state buffer."""
    d, p, mat, bck, terms, rec = _restart_setup()
    nx, nz = p["nx"], p["nz"]
    su, sw, s_full = O.psv_run("f32", nx, nz, p["npml"], 1, mat, bck, terms, rec, rec, 60)
    su1, sw1, s_half = O.psv_run("f32", nx, nz, p["npml"], 1, mat, bck, terms, rec, rec, 25)
    su2, sw2, s_end = O.psv_run("f32", nx, nz, p["npml"], 1, mat, bck, terms, rec, rec, 35, it0=25,
                                state=s_half)
    np.testing.assert_array_equal(s_full, s_end)
    np.testing.assert_array_equal(su, np.concatenate([su1, su2]))
