"""Box-source generator, CPU side: the oracle's restatement of ntde_line
(PD/source/source_line.cpp) against the golden vectors made by running the
reference program itself (tests/golden/line_source_ref.npz, made by
tests/golden/make_line_source.py), properties of the generator, and the
product's host entry points (radiation coefficients, plane origin)."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import fd23_oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "line_source_ref.npz")
# the oracle gathers the closed form per power of t, the reference evaluates
# it term by term: the two differ by rounding (measured <= 2e-10 of a
# point's largest value over these cases)
RTOL = 1e-8


def _load():
    z = np.load(GOLD)
    return z, json.loads(bytes(z["meta"]).decode())


def _wavelet(m):
    kv = dict(w.split("=") for w in m["stf"].split())
    if kv["sourcetime"].lower().startswith("t"):
        return O.trapezoid(m["dt"], float(kv["trap1"]), float(kv["trap2"]), float(kv["trap3"]))
    return O.gaussian(m["dt"], int(float(kv["alpha"])))


def _oracle(m, it0=0, nf=None):
    bw, o = m["bw"], O.box_plane_origin(m["bw"])
    a = O.line_source_coefs(*m["mech"])
    return O.line_source_planes(bw + 8, bw + 8, o, o, m["h"], m["dt"], m["vp"], m["vs"], m["den"], a,
                                _wavelet(m), it0, m["nt"] if nf is None else nf)


def _close(got, ref, scale):
    """equal NaN positions; elsewhere |got - ref| <= RTOL * scale"""
    np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))
    f = ~np.isnan(ref)
    d = np.abs(got - ref)[f]
    assert d.max(initial=0.0) <= RTOL * scale, d.max() / scale


@pytest.mark.parametrize("name", ["gauss_bw8", "trap_bw9", "nan_bw12", "long_bw16"])
def test_oracle_matches_reference_program(name):
    z, meta = _load()
    m = meta[name]
    P = _oracle(m)
    n = m["bw"] + 8
    assert P.shape == (m["nt"], 2, n, n)
    # NaN mask of the whole output (cells within one step of the source at t = 0)
    nan = np.unpackbits(z[name + "_nan"])[:P.size].reshape(P.shape).astype(bool)
    np.testing.assert_array_equal(np.isnan(P), nan)
    frames = z[name + "_frames"]
    stride = max(10, m["nt"] // 20)
    _close(P[::stride], frames, np.nanmax(np.abs(frames)))
    for (cx, cz), ser in zip(z[name + "_cells"], z[name + "_series"]):
        got = P[:, :, cz, cx]
        _close(got, ser, np.nanmax(np.abs(ser)) if np.isfinite(ser).any() else 1.0)
    # h / (vp dt) < 1 / 0.354 puts the nearest points within one step of the source
    assert nan.any() == (name in ("nan_bw12", "long_bw16"))


def test_oracle_against_live_reference(tmp_path):
    """Where the reference sources are present, build ntde_line and compare a
    case outside the fixtures (rectangular mechanism, trapezoid, bw 20)."""
    from oracle import build_ref
    exe = build_ref.build()
    if exe is None:
        pytest.skip("reference sources not present")
    bw, nt, h, dt, vp, vs, den = 20, 260, 4.0, 5e-4, 3200.0, 1800.0, 2.2
    stf = "sourcetime=trapezoid trap1=0.006 trap2=0.004 trap3=0.01"
    mech = (75, 20, 110, 300)
    par = (f"usebox=1 usepunch=0 ngpu=1\nnx=128 nz=128 nt={nt} h={h} dt={dt}\n"
           f"srcden={den} srcsvel={vs} srcpvel={vp} sourcefile=pl.bin bw={bw}\n{stf}\n"
           f"strike={mech[0]} dip={mech[1]} rake={mech[2]} azimuth={mech[3]}\n"
           f"xs=64 zs=64 npml=20 pml_dt={dt} pml_v=600 pml_r=1e-11 pml_fc=15\n"
           "itrecord=1 output=out nrec=1 ixrec0=10 izrec0_u=0 izrec0_w=0 idxrec=1 idzrec=0\n"
           "model=none.mdl ntsnap=100000\n")
    (tmp_path / "a.par").write_text(par)
    subprocess.check_call([exe, "par=a.par"], cwd=tmp_path, stdout=subprocess.DEVNULL)
    n = bw + 8
    ref = np.fromfile(tmp_path / "pl.bin", dtype=np.float64).reshape(nt, 2, n, n)
    m = dict(bw=bw, nt=nt, h=h, dt=dt, vp=vp, vs=vs, den=den, stf=stf, mech=mech)
    P = _oracle(m)
    scale = np.abs(ref).max(axis=0, keepdims=True)
    _close(P / np.where(scale > 0, scale, 1), ref / np.where(scale > 0, scale, 1), 1.0)


def _small(nf=80, src=None, it0=0, px=10, pz=7, ox=-5, oz=-3):
    a = O.line_source_coefs(30, 50, 70, 10)
    if src is None:
        src = O.gaussian(4e-4, -6)
    return O.line_source_planes(px, pz, ox, oz, 5.0, 4e-4, 3000.0, 1700.0, 2.5, a, src, it0, nf)


def test_generator_properties():
    src = O.gaussian(4e-4, -6)
    full = _small(80, src)
    # frames it0 .. it0+n-1 are the same frames of a run from 0
    np.testing.assert_array_equal(_small(30, src, it0=50), full[50:])
    # a one-tap wavelet of 1 gives the Green's function itself; the
    # convolution is linear in the wavelet and shifts with it
    g = _small(80, np.array([1.0]))
    two = _small(80, np.array([0.0, 0.0, 2.0]))
    np.testing.assert_allclose(two[2:], 2.0 * g[:-2], rtol=0, atol=0)
    assert not np.any(two[:2])
    s1, s2 = src, np.roll(src, 3) * 0.5
    np.testing.assert_allclose(_small(80, s1 + s2), _small(80, s1) + _small(80, s2), rtol=1e-12,
                               atol=1e-12 * np.abs(full).max())
    # nothing arrives before the P wave: a point's samples are zero up to
    # floor(R / vp / dt) (the arrival sample itself is evaluated)
    h, dt, vp = 5.0, 4e-4, 3000.0
    for (p, q) in ((0, 0), (9, 6), (4, 2)):
        x, zz = ((-5 + p) + 0.5) - 0.25, (-3 + q) + 0.25
        na = int(np.floor(np.hypot(x * h, zz * h) / vp / dt))
        assert not np.any(g[:na, 0, q, p])


def test_product_host_helpers_match_oracle():
    F = pytest.importorskip("fd23_gb300")
    try:
        F.lib()
    except ImportError:
        pytest.skip("library not built")
    for mech in ((30, 60, 90, 0), (10, 45, 30, 75), (200, 35, -60, 110), (0, 90, 0, 0)):
        np.testing.assert_array_equal(F.line_source_coefs(*mech), O.line_source_coefs(*mech))
    for bw in (8, 9, 16, 31, 32):
        assert F.line_plane_origin(bw) == O.box_plane_origin(bw)
        # the plane's cell 4 + bw//2 ... is the box's centre column: box cell i
        # at plane i + 4 is (bw + 1)/2 + 1 - bw + i cells from the source
        assert F.line_plane_origin(bw) + 4 == (bw + 1) // 2 + 1 - bw
    # argument errors need no GPU
    d = F.line_desc(16, 16, -7, -7, 5.0, 4e-4, 3000.0, 1700.0, 2.5, (1, 0, 0))
    src = np.ones(3)
    with pytest.raises(F.Fd23Error) as e:
        F.line_source_planes(F.line_desc(0, 16, -7, -7, 5.0, 4e-4, 3000.0, 1700.0, 2.5, (1, 0, 0)), src, 0, 4)
    assert e.value.status == F.ERR_ARG
    with pytest.raises(F.Fd23Error) as e:
        F.line_source_planes(F.line_desc(16, 16, -7, -7, 5.0, 4e-4, 0.0, 1700.0, 2.5, (1, 0, 0)), src, 0, 4)
    assert e.value.status == F.ERR_ARG
    with pytest.raises(F.Fd23Error) as e:
        F.line_source_planes(d, np.ones(8193), 0, 4)
    assert e.value.status == F.ERR_ARG


def test_late_arrivals_are_zero():
    """Points whose P arrival falls after the last frame are zero (the
    reference writes past its arrays there); frames that end just after an
    arrival carry it."""
    a = O.line_source_coefs(30, 50, 70, 10)
    src = O.gaussian(4e-4, -6)
    h, dt, vp = 5.0, 4e-4, 3000.0
    # a plane 40 .. 47 cells right of the source: R/vp/dt >= 166 steps
    far = O.line_source_planes(8, 4, 40, -2, h, dt, vp, 1700.0, 2.5, a, src, 0, 150)
    assert not np.any(far)
    late = O.line_source_planes(8, 4, 40, -2, h, dt, vp, 1700.0, 2.5, a, src, 0, 260)
    assert np.any(late[200:]) and not np.any(late[:150])
