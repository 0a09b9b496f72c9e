"""Hybrid box on the GPU: bit-exact parity with the oracle's box run (FP32 and
FP64, fused and two-pass sweeps), the self-consistency property at a size
with many sweep work items, split runs, and argument errors."""
import numpy as np
import pytest

from oracle import fd23_oracle as O
from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")


def _solver(c, prec, kernel, source=True):
    s = F.Solver("psv", c.nx, c.nz, c.npml, c.h, c.dt, prec=prec, topabsorb=c.topabsorb,
                 kernel=kernel, **c.pml)
    s.set_model(c.vp, c.vs, c.den)
    if source:
        s.set_source(c.kind, c.xs, c.zs, c.m, c.src, c.nt)
    return s


def _receivers(c, extra_x, extra_z):
    rx = np.concatenate([c.rx, extra_x]).astype(np.int32)
    rz = np.concatenate([c.rz, extra_z]).astype(np.int32)
    return rx, rz


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("kernel", ["fused", "twopass"])
# one-CTA kernels (small boxes), multi-CTA kernels (odd and even widths)
@pytest.mark.parametrize("box", [(70, 30, 64, 56), (20, 14, 130, 101), (16, 12, 128, 100)])
def test_box_parity_with_oracle(prec, kernel, box):
    """Box driven by the ring field of a run in another model (so the residual
    field is far from zero), with the grid's own point source outside the box
    and receivers on every field, in the rings, the box interior and outside."""
    nx, nz, nt = 160, 120, 60
    c = Case("psv", nx, nz, npml=12, nt=nt, xs=30 if box[0] > 30 else 10, zs=8, seed=7)
    x0, z0, bx, bz = box
    # incident field: a run in a different (seeded) model with its source in the box
    ci = Case("psv", nx, nz, npml=12, nt=nt, xs=100, zs=55, seed=21)
    inc, _ = O.psv_ring_history("f64", nx, nz, 12, 0, ci.mat, ci.bck, ci.terms, nt, box)
    dt_ = np.float64 if prec == "f64" else np.float32
    inc = inc.astype(dt_)
    rmat = np.ascontiguousarray(c.mat[:, z0:z0 + bz, x0:x0 + bx])
    # receivers: the standard line, plus cells on the rings and inside the box
    ex = np.array([x0, x0 + 3, x0 + 5, x0 + 20, x0 + bx - 1, x0 + bx - 6, x0 + 30])
    ez = np.array([z0, z0 + 10, z0 + 6, z0 + 2, z0 + 30, z0 + bz - 7, z0 + 25])
    rx, rz = _receivers(c, ex, ez)
    rec = rx + rz * nx
    rf = np.repeat(np.arange(5, dtype=np.int32), len(rec))
    ri = np.tile(rec, 5)
    seis_o, st_o, r_o = O.psv_box_run(prec, nx, nz, c.npml, 0, c.mat, c.bck, c.terms, rf, ri, nt,
                                      box, rmat, inc)
    assert np.abs(r_o).max() > 0
    s = _solver(c, prec, kernel)
    for f in range(5):
        s.set_receivers(f, rx, rz)
    s.set_box(x0, z0, bx, bz)  # cut of the grid material, = rmat
    s.set_box_incident(inc, 0)
    s.run(nt, 1)
    for f in range(5):
        np.testing.assert_array_equal(s.seismograms(f), seis_o[:, f * len(rec):(f + 1) * len(rec)],
                                      err_msg="field %d" % f)
    np.testing.assert_array_equal(s.get_state(), st_o)
    np.testing.assert_array_equal(s.get_box_state(), r_o)
    s.close()


@pytest.mark.parametrize("kernel", ["fused", "twopass"])
def test_box_reproduces_recorded_run(kernel):
    """The ring field of a GPU run, recorded with stress and velocity receivers
    on the ring cells, drives a box run without the source: outside the box
    interior the wavefields and the surface seismograms equal the recorded
    run bit for bit, and the residual field stays zero."""
    nx, nz, nt = 700, 400, 120
    c = Case("psv", nx, nz, npml=20, nt=nt, xs=350, zs=100, seed=9, wavelet=("gauss", -6))
    x0, z0, bx, bz = 200, 40, 300, 200
    rix, riz = F.box_ring_cells(x0, z0, bx, bz)
    nring = len(rix)
    plain = _solver(c, "f32", kernel)
    for f in range(5):
        plain.set_receivers(f, np.concatenate([c.rx, rix]), np.concatenate([c.rz, riz]))
    plain.run(nt, 1)
    nr = len(c.rx)
    rec = [plain.seismograms(f) for f in range(5)]
    inc = np.zeros((nt, 5, nring), np.float32)
    for f in (0, 1):  # velocities before the step = after the previous one
        inc[1:, f] = rec[f][:-1, nr:]
    for f in (2, 3, 4):  # stresses after the step's stress update
        inc[:, f] = rec[f][:, nr:]
    st_plain = plain.get_state()
    plain.close()

    b = _solver(c, "f32", kernel, source=False)
    b.set_receivers(0, c.rx, c.rz)
    b.set_receivers(1, c.rx, c.rz)
    b.set_box(x0, z0, bx, bz)
    b.set_box_incident(inc, 0)
    b.run(nt, 1)
    keep = np.ones((nz, nx), bool)
    keep[z0 + 4:z0 + bz - 4, x0 + 4:x0 + bx - 4] = False
    out = keep[c.rz, c.rx]
    for f in (0, 1):
        np.testing.assert_array_equal(b.seismograms(f)[:, out], rec[f][:, :nr][:, out])
    st = b.get_state()
    n = nx * nz
    for f in range(5):
        np.testing.assert_array_equal(st[f * n:(f + 1) * n].reshape(nz, nx)[keep],
                                      st_plain[f * n:(f + 1) * n].reshape(nz, nx)[keep])
    np.testing.assert_array_equal(st[5 * n:], st_plain[5 * n:])
    assert not np.any(b.get_box_state())
    b.close()


def test_box_split_runs_and_state():
    """run(a) + run(b) equals run(a+b); the residual field survives a box
    state round trip; the incident window may be loaded piecewise."""
    nx, nz, nt = 200, 140, 50
    c = Case("psv", nx, nz, npml=12, nt=nt, xs=40, zs=10, seed=2)
    ci = Case("psv", nx, nz, npml=12, nt=nt, xs=110, zs=60, seed=3)
    box = (80, 40, 48, 40)
    inc, _ = O.psv_ring_history("f32", nx, nz, 12, 0, ci.mat, ci.bck, ci.terms, nt, box)
    one = _solver(c, "f32", "fused")
    one.set_receivers(0, c.rx, c.rz)
    one.set_box(*box)
    one.set_box_incident(inc, 0)
    one.run(nt, 2)
    two = _solver(c, "f32", "fused")
    two.set_receivers(0, c.rx, c.rz)
    two.set_box(*box)
    two.set_box_incident(inc[:20], 0)
    two.run(20, 2)
    with pytest.raises(F.Fd23Error):  # step 20 not loaded yet
        two.run(1, 2)
    r = two.get_box_state()
    two.set_box_state(np.zeros_like(r))
    two.set_box_state(r)
    two.set_box_incident(inc[20:], 20)
    two.run(nt - 20, 2)
    np.testing.assert_array_equal(two.seismograms(0), one.seismograms(0))
    np.testing.assert_array_equal(two.get_state(), one.get_state())
    np.testing.assert_array_equal(two.get_box_state(), one.get_box_state())
    # removing the box returns to the plain sweep
    one.set_box(0, 0, 0, 0)
    one.run(2, 1)
    one.close()
    two.close()


def test_box_argument_errors():
    c = Case("psv", 120, 90, npml=10, nt=10)
    s = _solver(c, "f32", "fused")
    with pytest.raises(F.Fd23Error):
        s.set_box(110, 10, 20, 20)  # outside the grid
    with pytest.raises(F.Fd23Error):
        s.set_box(10, 10, 15, 30)  # below the 16-cell minimum
    with pytest.raises(F.Fd23Error):
        s.set_box_incident(np.zeros((1, 5, 10), np.float32), 0)  # no box yet
    with pytest.raises(F.Fd23Error) as e:
        s.set_box_incident(np.zeros((1, 5, 10), np.float32), 0, wait=False)
    assert e.value.status == F.ERR_ORDER
    s.set_box(10, 10, 40, 30)
    with pytest.raises(F.Fd23Error) as e:
        s.run(1, 1)  # incident field not loaded
    assert e.value.status == F.ERR_ORDER
    # an asynchronous upload of 3 steps covers 3 steps only
    nring = sum(F.box_ring_size(40, 30))
    s.set_box_incident(np.zeros((3, 5, nring), np.float32), 0, wait=False)
    with pytest.raises(F.Fd23Error) as e:
        s.run(4, 1)
    assert e.value.status == F.ERR_ORDER
    s.run(3, 1)
    s.sync()
    s.close()
    sh = F.Solver("sh", 120, 90, 10, c.h, c.dt, prec="f32", **c.pml)
    with pytest.raises(F.Fd23Error) as e:
        sh.set_box(10, 10, 40, 30)
    assert e.value.status == F.ERR_UNSUPPORTED
    sh.close()
    b16 = F.Solver("psv", 120, 90, 10, c.h, c.dt, prec="bf16", **c.pml)
    b16.set_model(c.vp, c.vs, c.den)
    with pytest.raises(F.Fd23Error) as e:
        b16.set_box(10, 10, 40, 30)
    assert e.value.status == F.ERR_UNSUPPORTED
    b16.close()


def test_array_size_checks():
    """Host arrays of the wrong size are refused before the C side reads them."""
    c = Case("psv", 120, 90, npml=10, nt=10)
    s = _solver(c, "f32", "fused")
    with pytest.raises(ValueError):
        s.set_model(c.vp[:45], c.vs, c.den)
    with pytest.raises(ValueError):
        s.set_material(c.mat[:3])
    with pytest.raises(ValueError):
        s.set_receivers(0, c.rx, c.rz[:-1])
    with pytest.raises(ValueError):
        s.set_box(10, 10, 40, 30, np.zeros((5, 30, 39)))
    s.set_box(10, 10, 40, 30)
    with pytest.raises(ValueError):
        s.set_box_incident(np.zeros((2, 5, 7), np.float32), 0)
    s.close()


def test_box_incident_async_upload():
    """fd23_set_box_incident_async (chunks of 64 steps on a copy stream, each
    box step waiting only for its chunk) gives the results of the waiting
    upload: one run over more than one chunk, a second upload into the same
    buffer while the first run's work may still be queued, and split runs."""
    nx, nz, nt = 200, 140, 150
    c = Case("psv", nx, nz, npml=12, nt=nt, xs=40, zs=10, seed=4)
    ci = Case("psv", nx, nz, npml=12, nt=nt, xs=110, zs=60, seed=5)
    box = (80, 40, 48, 40)
    inc, _ = O.psv_ring_history("f32", nx, nz, 12, 0, ci.mat, ci.bck, ci.terms, nt, box)
    out = {}
    for wait in (True, False):
        s = _solver(c, "f32", "fused")
        s.set_receivers(0, c.rx, c.rz)
        s.set_box(*box)
        s.set_box_incident(inc, 0, wait=wait)
        s.run(nt, 1)
        first = (s.seismograms(0), s.get_state(), s.get_box_state())
        # again from the start, the upload queued behind nothing or behind the reset
        s.reset()
        s.set_box(*box)
        s.set_box_incident(inc[:70], 0, wait=wait)
        s.run(70, 1)
        s.set_box_incident(inc[70:], 70, wait=wait)
        s.run(nt - 70, 1)
        second = (s.seismograms(0), s.get_state(), s.get_box_state())
        for a, b in zip(first, second):
            np.testing.assert_array_equal(a, b)
        out[wait] = first
        s.close()
    for a, b in zip(out[True], out[False]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_set_model_box_equals_host_path(prec):
    """fd23_set_model_box (material built on the device, the box homogenised
    towards the source material, the box material installed) gives the host
    path's results (fd23_build_material, fd23_box_material, set_material,
    set_box with bmat): the same number of replaced cells, and bit for bit the
    same seismograms, state and residual field of a box run.  The box
    straddles a layer boundary, so part of it takes the source material."""
    nx, nz, npml, nt = 260, 180, 12, 50
    c = Case("psv", nx, nz, npml=npml, nt=nt, xs=60, zs=10, seed=6)
    vp = np.full((nz, nx), 4.0)
    vp[90:, :] = 5.0
    vp[:, 200:] += 0.5  # a lateral step outside the box
    vs, den = vp / 1.73, 0.31 * vp ** 0.25 * 8.0
    x0, z0, bw = 110, 76, 32
    sv = (float(vp[z0 + 2, x0 + 2]), float(vs[z0 + 2, x0 + 2]), float(den[z0 + 2, x0 + 2]))
    mat, stab, rc = F.build_material("psv", vp, vs, den, c.h, c.dt)
    assert rc == 0
    mat, bmat, nrep = F.box_material(mat, x0, z0, bw, bw, *sv, c.dt, c.h)
    assert 0 < nrep < bw * bw
    ci = Case("psv", nx, nz, npml=npml, nt=nt, xs=120, zs=92, seed=23)
    box = (x0, z0, bw, bw)
    inc, _ = O.psv_ring_history("f64", nx, nz, npml, 0, ci.mat, ci.bck, ci.terms, nt, box)
    inc = inc.astype(np.float64 if prec == "f64" else np.float32)
    out = {}
    for path in ("host", "device"):
        s = F.Solver("psv", nx, nz, npml, c.h, c.dt, prec=prec, kernel="fused", **c.pml)
        if path == "host":
            s.set_material(mat)
            s.set_box(*box, bmat=bmat)
        else:
            n_dev, bmat_dev = s.set_model_box(vp, vs, den, *box, *sv)
            assert n_dev == nrep
            np.testing.assert_array_equal(bmat_dev, bmat)
        s.set_source(c.kind, c.xs, c.zs, c.m, c.src, nt)
        for f in range(5):
            s.set_receivers(f, np.array([20, 111, 126, 140, 250], np.int32), np.array([0, 77, 92, 100, 5], np.int32))
        s.set_box_incident(inc, 0)
        s.run(nt, 1)
        out[path] = [s.seismograms(f) for f in range(5)] + [s.get_state(), s.get_box_state()]
        s.close()
    assert np.abs(out["device"][-1]).max() > 0
    for a, b in zip(out["host"], out["device"]):
        np.testing.assert_array_equal(a, b)
