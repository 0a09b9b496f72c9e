"""The oracle pinned to the reference programs' own host code.

tests/golden/ref_pins.npz holds what the reference's host code computes when
it is built from its sources here (oracle/build_ref.py,
oracle/ref_setup_harness.cpp; generator tests/golden/make_ref_pins.py):

* FP64 P-SV (PSV/psv_clean_double): material, CPML coefficients, box ring
  lists, box material and the box's incident field (setboxsource) --
  bit-exact; the residual step (fd/fd.cpp step_stress_r, step_velocity_r) --
  within FP64 round-off, because the oracle (like the reference's GPU
  build) accumulates with fused multiply-adds where the host loop rounds
  every product.
* FP32 P-SV (PSV/clean_nobox) and SH: material and CPML coefficients within
  a few FP32 ulps.  The reference builds them in float arithmetic; this build
  builds every coefficient in FP64 and rounds once (the same formulas, the
  same edge rules: a logic difference would show as an O(1) error).
* SH host step (SH/fd/fd.cpp:43,121) from a seeded state: within 1 FP32 ulp
  of each field's largest value on every cell at least 6 from the edges (the
  host loop's stencil order ignores the top edge, PD/fd/fd.cpp:138-style,
  which changes rows within 6 of it), CPML cells included.

And the FP32 restart states (PSV/clean_nobox/TEST/tt): the residual at step
500 is the reference run's own FP32 rounding noise -- the reference state is
as far from the FP64 solution as any FP32 run here is (with or without fused
multiply-adds), so no FP32 arithmetic order reproduces it more closely.
"""
import json
import os

import numpy as np
import pytest

from oracle import fd23_oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PML = dict(pml_dt=0.005, pml_r=1e-11, pml_v=30.0, pml_fc=2.0)


@pytest.fixture(scope="module")
def pins():
    return np.load(os.path.join(GOLD, "ref_pins.npz"))


def _ulps(a, b):
    """largest distance in FP32 units in the last place"""
    ia = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    ib = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    # map the sign-magnitude order onto a line
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return int(np.max(np.abs(ia - ib)))


# ------------------------------------------------------------- FP64 P-SV
@pytest.mark.parametrize("key", ["pd20", "pd17"])
def test_fp64_material_and_cpml_bit_exact(pins, key):
    vp, vs, den = pins[key + "_in"].astype(np.float64)
    nx, nz, npml = [int(v) for v in pins[key + "_geom"][:3]]
    h, dt = pins[key + "_hdt_src"][:2]
    mat, _, rc = O.psv_material(vp, vs, den, h, dt)
    assert rc == 0
    np.testing.assert_array_equal(mat, pins[key + "_mat"])
    bck = O.cpml_psv(nx, nz, npml, **PML)
    np.testing.assert_array_equal(np.asarray(bck).ravel(), pins[key + "_bck"])


@pytest.mark.parametrize("key", ["pd20", "pd17"])
def test_box_rings_material_incident_bit_exact(pins, key):
    nx, nz, npml, xs, zs, bw = [int(v) for v in pins[key + "_geom"]]
    h, dt, srcvp, srcvs, srcden = pins[key + "_hdt_src"]
    # PD/box/box.cpp:30-40: the box of width bw around (xs, zs)
    idxend = (bw + 1) // 2
    x0, z0 = xs + idxend + 1 - bw, zs + idxend + 1 - bw
    nsub, nadd, sx, sz = [int(v) for v in pins[key + "_box_head"]]
    assert (sx, sz) == (x0, z0)
    g, r, ns = O.box_rings(nx, x0, z0, bw, bw)
    assert ns == nsub and len(g) == nsub + nadd
    np.testing.assert_array_equal(r, np.concatenate([pins[key + "_r_sub"], pins[key + "_r_add"]]))
    np.testing.assert_array_equal(g, np.concatenate([pins[key + "_a_sub"], pins[key + "_a_add"]]))
    full, rmat, nrep = O.box_material(pins[key + "_mat"], x0, z0, bw, bw, srcvp, srcvs, srcden, dt, h)
    np.testing.assert_array_equal(rmat, pins[key + "_bmat"])
    # pd20: no box cell is in the source material; pd17: its upper half is
    assert (nrep == bw * bw) if key == "pd20" else (0 < nrep < bw * bw)
    planes, sfield = pins[key + "_planes"], pins[key + "_sfield"]
    for k in range(1, planes.shape[0]):
        inc = O.box_incident_from_displacement(bw, bw, dt, rmat, planes[k - 1, 0], planes[k - 1, 1],
                                               planes[k, 0], planes[k, 1])
        # the reference fills the whole bw x bw field; the ring cells are used
        np.testing.assert_array_equal(inc, sfield[k - 1].reshape(5, -1)[:, r])


@pytest.mark.parametrize("key", ["pd20", "pd17"])
def test_box_residual_step(pins, key):
    bw = int(pins[key + "_geom"][5])
    out = O.box_residual_step(pins[key + "_bmat"], pins[key + "_resid_in"])
    ref = pins[key + "_resid_out"]
    # FP64 round-off of a fused against an unfused accumulation
    assert np.max(np.abs(out - ref)) <= 1e-15 * np.max(np.abs(ref))
    # cells outside 4 .. bw-5 are not updated by either
    edge = np.ones((bw, bw), bool)
    edge[4:bw - 4, 4:bw - 4] = False
    np.testing.assert_array_equal(out[:, edge], pins[key + "_resid_in"][:, edge])


# ------------------------------------------------------------- FP32 set-up
@pytest.mark.parametrize("key", ["pn_restart", "pn_layered"])
def test_fp32_psv_setup_within_float_rounding(pins, key):
    vp, vs, den = pins[key + "_in"].astype(np.float64)
    nx, nz, npml = [int(v) for v in pins[key + "_geom"]]
    h, dt = pins[key + "_hdt"]
    mat, _, rc = O.psv_material(vp, vs, den, h, dt)
    assert rc == 0
    ref = pins[key + "_mat"]
    for m in range(5):
        # lam = vp^2 rho - 2 mu in float cancels: a few ulps
        assert _ulps(mat[m].astype(np.float32), ref[m]) <= 8, m
    bck = np.asarray(O.cpml_psv(nx, nz, npml, **PML)).ravel().astype(np.float32)
    # b, c, k are O(1) or below: absolute FP32 round-off of 1
    assert np.max(np.abs(bck.astype(np.float64) - pins[key + "_bck"])) <= 2.0 ** -23


def test_sh_setup_within_float_rounding(pins):
    vp, vs, den = pins["sh_in"].astype(np.float64)
    nx, nz, npml = [int(v) for v in pins["sh_geom"]]
    h, dt = pins["sh_hdt"]
    mat, _, rc = O.sh_material(vs, den, h, dt)
    assert rc == 0
    for m in range(3):  # MUX (harmonic with the next cell, row wrap), MUZ, BV
        assert _ulps(mat[m].astype(np.float32), pins["sh_mat"][m]) <= 2, m
    bck = np.asarray(O.cpml_sh(nx, nz, npml, **PML)).ravel().astype(np.float32)
    assert np.max(np.abs(bck.astype(np.float64) - pins["sh_bck"])) <= 2.0 ** -23


def test_sh_host_step_interior(pins):
    nx, nz, npml = [int(v) for v in pins["sh_geom"]]
    n = nx * nz
    st = np.zeros(O.sh_state_size(nx, nz, npml), np.float32)
    st[:3 * n] = pins["sh_state_in"].ravel()
    no_src = (np.zeros(0, np.int32), np.zeros(0, np.int64), np.zeros((0, 1)))
    # the reference's own material and CPML, so the step alone is compared
    _, s = O.sh_run("f32", nx, nz, npml, 0, pins["sh_mat"].astype(np.float64),
                    pins["sh_bck"].astype(np.float64), no_src, np.zeros(0, np.int64), 1, state=st)
    got = s[:3 * n].reshape(3, nz, nx).astype(np.float64)
    ref = pins["sh_state_out"].astype(np.float64)
    m = 6
    for f in range(3):  # V, Tx, Tz
        ulp = np.spacing(np.float32(np.max(np.abs(ref[f]))))
        assert np.max(np.abs(got[f, m:nz - m, m:nx - m] - ref[f, m:nz - m, m:nx - m])) <= ulp, f


# ------------------------------------------------------- FP32 restart states
def _restart():
    d = np.load(os.path.join(GOLD, "psv_fp32_restart.npz"))
    p = json.loads(str(d["params"]))
    nx, nz, h, dt = p["nx"], p["nz"], p["h"], p["dt"]
    vp, vs, den = (np.full((nz, nx), p[k]) for k in ("vp", "vs", "den"))
    mat, _, _ = O.psv_material(vp, vs, den, h, dt)
    bck = O.cpml_psv(nx, nz, p["npml"], p["pml_dt"], p["pml_r"], p["pml_v"], p["pml_fc"])
    src = O.gaussian(dt, p["alpha"])
    m = O.moment_psv(p["strike"], p["dip"], p["rake"], p["azimuth"])
    terms = O.source_terms("psv", p["stype"], nx, p["xs"], p["zs"], m, h, dt, src, 1000)
    return d, p, mat, bck, terms


def test_fp32_restart_residual_is_fp32_noise():
    d, p, mat, bck, terms = _restart()
    nx, nz, npml, top = p["nx"], p["nz"], p["npml"], p["topabsorb"]
    n = nx * nz
    runs = {}
    for prec in ("f64", "f32", "f32nf"):
        _, _, s = O.psv_run(prec, nx, nz, npml, top, mat, bck, terms, [], [], 500)
        runs[prec] = s.astype(np.float64)
    ref = d["state000499"].astype(np.float64)
    for f in (0, 1):  # U, W: the fields with the largest residual (~2e-5)
        sl = slice(f * n, (f + 1) * n)
        ref_vs_f64 = O.rel_l2(ref[sl], runs["f64"][sl])
        f32_vs_f64 = O.rel_l2(runs["f32"][sl], runs["f64"][sl])
        nf_vs_f64 = O.rel_l2(runs["f32nf"][sl], runs["f64"][sl])
        # the reference's FP32 state is no farther from the FP64 solution than
        # FP32 rounding puts any FP32 run, with or without fused multiply-adds
        assert ref_vs_f64 <= 1.5 * min(f32_vs_f64, nf_vs_f64), (f, ref_vs_f64, f32_vs_f64, nf_vs_f64)
        # and the residual against it is of that same size, not smaller
        # without fused multiply-adds (a -G build would be no closer)
        assert O.rel_l2(runs["f32nf"][sl], ref[sl]) > 0.5 * O.rel_l2(runs["f32"][sl], ref[sl])
