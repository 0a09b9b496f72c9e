"""Box-source generator on the GPU: the displacement planes equal the
oracle's bit for bit (and so the reference program's to its rounding), over
odd and rectangular planes, NaN points, frame offsets, wavelet lengths and a
run longer than one frame chunk; and a hybrid box driven by the generator on
the device equals the same box driven through the host path (planes ->
setboxsource -> incident upload) and the oracle's box run."""
import json
import os

import numpy as np
import pytest

from oracle import fd23_oracle as O
from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")

GOLD = os.path.join(os.path.dirname(__file__), "golden", "line_source_ref.npz")


def _planes(px, pz, ox, oz, h, dt, vp, vs, den, mech, src, it0, nf):
    a = O.line_source_coefs(*mech)
    ref = O.line_source_planes(px, pz, ox, oz, h, dt, vp, vs, den, a, src, it0, nf)
    got = F.line_source_planes(F.line_desc(px, pz, ox, oz, h, dt, vp, vs, den, F.line_source_coefs(*mech)),
                               src, it0, nf)
    return got, ref


CASES = [
    # px, pz, ox, oz, h, dt, vp, vs, den, mechanism, wavelet, it0, nframes
    (16, 16, -7, -7, 5.0, 4e-4, 3000.0, 1730.0, 2500.0, (30, 60, 90, 0), ("g", -8), 0, 100),
    (17, 17, -8, -8, 5.0, 4e-4, 3000.0, 1730.0, 2500.0, (10, 45, 30, 75), ("t", 0.004, 0.008, 0.006), 0, 300),
    (20, 20, -9, -9, 1.0, 4e-4, 3000.0, 1730.0, 2500.0, (0, 90, 0, 20), ("g", 5), 0, 200),      # NaN points
    (37, 23, -20, -3, 4.0, 5e-4, 3500.0, 2000.0, 2.4, (45, 70, 150, 300), ("g", -20), 0, 400),  # rectangle
    (29, 31, -60, 12, 5.0, 4e-4, 3000.0, 1700.0, 2.5, (200, 35, -60, 110), ("g", -6), 250, 90),  # offset
    (12, 9, -6, -4, 5.0, 4e-4, 3000.0, 1700.0, 2.5, (80, 10, 20, 30), ("one",), 0, 150),           # one tap
]


def _wavelet(w, dt):
    if w[0] == "g":
        return O.gaussian(dt, w[1])
    if w[0] == "t":
        return O.trapezoid(dt, *w[1:])
    return np.array([0.7])


@pytest.mark.parametrize("case", range(len(CASES)))
def test_planes_equal_oracle(case):
    px, pz, ox, oz, h, dt, vp, vs, den, mech, w, it0, nf = CASES[case]
    got, ref = _planes(px, pz, ox, oz, h, dt, vp, vs, den, mech, _wavelet(w, dt), it0, nf)
    assert got.shape == (nf, 2, pz, px)
    np.testing.assert_array_equal(got, ref)  # NaN at the same places
    assert np.nanmax(np.abs(got)) > 0
    # NaN iff a point lies within one step's travel of the source (0/0 at t = 0)
    # and frame 0 is within the wavelet's reach of the frames asked for
    pp, qq = np.meshgrid(np.arange(px), np.arange(pz))
    near = min(np.hypot(((ox + pp) + 0.5 - 0.25) * h, ((oz + qq) + 0.25) * h).min(),
               np.hypot(((ox + pp) - 0.25) * h, ((oz + qq) - 0.25) * h).min()) / vp / dt < 1.0
    ntap = (len(_wavelet(w, dt)) + 31) // 32 * 32
    assert np.isnan(got).any() == (near and it0 < ntap)
    assert np.isnan(got).any() == (case in (2, 3))


def test_planes_match_reference_fixture():
    z = np.load(GOLD)
    meta = json.loads(bytes(z["meta"]).decode())
    for name, m in meta.items():
        kv = dict(w.split("=") for w in m["stf"].split())
        if kv["sourcetime"].lower().startswith("t"):
            src = O.trapezoid(m["dt"], float(kv["trap1"]), float(kv["trap2"]), float(kv["trap3"]))
        else:
            src = O.gaussian(m["dt"], int(float(kv["alpha"])))
        bw = m["bw"]
        o = F.line_plane_origin(bw)
        d = F.line_desc(bw + 8, bw + 8, o, o, m["h"], m["dt"], m["vp"], m["vs"], m["den"],
                        F.line_source_coefs(*m["mech"]))
        got = F.line_source_planes(d, src, 0, m["nt"])
        nan = np.unpackbits(z[name + "_nan"])[:got.size].reshape(got.shape).astype(bool)
        np.testing.assert_array_equal(np.isnan(got), nan)
        fr = z[name + "_frames"]
        sel = got[::max(10, m["nt"] // 20)]
        ok = ~np.isnan(fr)
        assert np.abs(sel - fr)[ok].max() <= 1e-8 * np.abs(fr[ok]).max(), name


def test_planes_across_chunks():
    """More frames than one device chunk holds (8192): the second chunk's
    window and history line up with the first's."""
    got, ref = _planes(3, 2, -1, -1, 5.0, 4e-4, 3000.0, 1700.0, 2.5, (30, 40, 50, 60), O.gaussian(4e-4, -6),
                       0, 8300)
    np.testing.assert_array_equal(got, ref)


def _box_setup(prec, nx=160, nz=120, nt=80, bw=40, xs=80, zs=60, npml=12, seed=5):
    c = Case("psv", nx, nz, npml=npml, nt=nt, seed=seed)
    srcvp, srcvs, srcden = 4.5, 2.6, 3.7
    x0 = xs + (bw + 1) // 2 + 1 - bw
    z0 = zs + (bw + 1) // 2 + 1 - bw
    mat, bmat, _ = F.box_material(c.mat, x0, z0, bw, bw, srcvp, srcvs, srcden, c.dt, c.h)
    o = F.line_plane_origin(bw)
    mech = (30, 60, 90, 45)
    src = O.gaussian(c.dt, -4)
    desc = F.line_desc(bw + 8, bw + 8, o, o, c.h, c.dt, srcvp, srcvs, srcden, F.line_source_coefs(*mech))
    # host path: planes -> setboxsource per step
    pl = O.line_source_planes(bw + 8, bw + 8, o, o, c.h, c.dt, srcvp, srcvs, srcden, O.line_source_coefs(*mech),
                              src, 0, nt + 1)
    inc = np.stack([O.box_incident_from_displacement(bw, bw, c.dt, bmat, pl[i, 0], pl[i, 1], pl[i + 1, 0],
                                                     pl[i + 1, 1]) for i in range(nt)])
    return c, mat, bmat, (x0, z0, bw, bw), desc, src, inc


def _box_run(c, prec, kernel, mat, bmat, box, rx, rz, inc=None, line=None, nt=None):
    nt = c.nt if nt is None else nt
    s = F.Solver("psv", c.nx, c.nz, c.npml, c.h, c.dt, prec=prec, kernel=kernel, **c.pml)
    s.set_material(mat)
    for f in range(5):
        s.set_receivers(f, rx, rz)
    s.set_box(*box, bmat=bmat)
    if inc is not None:
        s.set_box_incident(inc.astype(s.dtype), 0)
    else:
        desc, src = line
        s.set_box_line_source(desc, src, bmat, 0, nt)
    s.run(nt, 1)
    out = [s.seismograms(f) for f in range(5)], s.get_state(), s.get_box_state()
    s.close()
    return out


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("kernel", ["fused", "twopass"])
def test_box_line_source_equals_host_path(prec, kernel):
    c, mat, bmat, box, desc, src, inc = _box_setup(prec)
    x0, z0, bx, bz = box
    rx = np.concatenate([c.rx, [x0 + 1, x0 + 6, x0 + bx // 2, x0 - 3, x0 + bx + 2]]).astype(np.int32)
    rz = np.concatenate([c.rz, [z0 + 2, z0 + 5, z0 - 2, z0 + bz // 2, z0 + 9]]).astype(np.int32)
    seis_h, st_h, r_h = _box_run(c, prec, kernel, mat, bmat, box, rx, rz, inc=inc)
    seis_d, st_d, r_d = _box_run(c, prec, kernel, mat, bmat, box, rx, rz, line=(desc, src))
    for a, b in zip(seis_d, seis_h):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(st_d, st_h)
    np.testing.assert_array_equal(r_d, r_h)
    assert np.abs(seis_d[0]).max() > 0  # the box's wave reached the receivers
    if prec == "f64" and kernel == "fused":
        rec = rx + rz * c.nx
        rf = np.repeat(np.arange(5, dtype=np.int32), len(rec))
        no_source = (np.zeros(0, np.int32), np.zeros(0, np.int64), np.zeros((0, 1)))
        seis_o, st_o, r_o = O.psv_box_run("f64", c.nx, c.nz, c.npml, 0, mat, c.bck, no_source, rf,
                                          np.tile(rec, 5), c.nt, box, bmat, inc)
        for f in range(5):
            np.testing.assert_array_equal(seis_d[f], seis_o[:, f * len(rec):(f + 1) * len(rec)])
        np.testing.assert_array_equal(st_d, st_o)
        np.testing.assert_array_equal(r_d, r_o)


def test_box_line_source_across_chunks():
    """8300 steps: the device generator's second chunk of steps continues the
    first (small grid and box so that the run is short)."""
    nt = 8300
    c, mat, bmat, box, desc, src, inc = _box_setup("f32", nx=64, nz=64, nt=nt, bw=16, xs=32, zs=32, npml=8,
                                                   seed=3)
    rx = np.array([2, 10, 30, 50, 61], np.int32)
    rz = np.array([0, 3, 12, 40, 60], np.int32)
    seis_h, st_h, r_h = _box_run(c, "f32", "fused", mat, bmat, box, rx, rz, inc=inc)
    seis_d, st_d, r_d = _box_run(c, "f32", "fused", mat, bmat, box, rx, rz, line=(desc, src))
    for a, b in zip(seis_d, seis_h):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(st_d, st_h)


def test_box_line_source_errors():
    c, mat, bmat, box, desc, src, inc = _box_setup("f32", nt=4)
    s = F.Solver("psv", c.nx, c.nz, c.npml, c.h, c.dt, prec="f32", **c.pml)
    s.set_material(mat)
    with pytest.raises(F.Fd23Error) as e:  # no box yet
        s.set_box_line_source(desc, src, bmat, 0, 4)
    assert e.value.status == F.ERR_ORDER
    s.set_box(*box, bmat=bmat)
    wrong = F.line_desc(desc.px + 1, desc.pz, desc.ox, desc.oz, desc.h, desc.dt, desc.vp, desc.vs, desc.den,
                        list(desc.a))
    with pytest.raises(F.Fd23Error) as e:
        s.set_box_line_source(wrong, src, bmat, 0, 4)
    assert e.value.status == F.ERR_ARG
    s.set_box_line_source(desc, src, bmat, 0, 4)
    s.run(4, 1)
    with pytest.raises(F.Fd23Error) as e:  # step 4 has no incident field
        s.run(1, 1)
    assert e.value.status == F.ERR_ORDER
    s.close()
