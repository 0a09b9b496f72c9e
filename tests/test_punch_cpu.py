"""usepunch (tile step windows), CPU side: the oracle's window builder
against the reference's SLIDE loops written out, the product's builder and
file reader against the oracle (bit for bit, both precisions, ragged grids,
odd values), and the oracle's windowed run against its plain run."""
import numpy as np
import pytest

from oracle import fd23_oracle as O
from tests.fd23_cases import Case

F = pytest.importorskip("fd23_gb300")


def _lib_or_skip():
    try:
        F.lib()
    except ImportError as e:
        pytest.skip(str(e))


def reference_slide(times, before, after, dt, elem):
    """PD/slide/cu_slide.cu:23-55 (elem f64) and PN/slide/cu_slide.cu (f32):
    read BDIMY = 16 rows of nx at a time, per BDIMX = 32 column tile take
    min / max from the 1E28 sentinels, then int((min - before)/dt) and
    int((max + after)/dt); scalars of the file's type throughout."""
    T = np.float64 if elem == "f64" else np.float32
    nz, nx = times.shape
    nxblock, nzblock = nx // 32, nz // 16
    first = np.zeros(nxblock * nzblock, np.int32)
    last = np.zeros(nxblock * nzblock, np.int32)
    b, a, d = T(before), T(after), T(dt)
    for k in range(nzblock):
        buf = np.asarray(times[k * 16:(k + 1) * 16], dtype=T).ravel()
        for i in range(nxblock):
            mn, mx = T(1e28), T(-1e28)
            for kk in range(16):
                for ii in range(32):
                    v = buf[kk * nx + i * 32 + ii]
                    mn = v if v < mn else mn
                    mx = v if mx < v else mx
            first[k * nxblock + i] = int((mn - b) / d)
            last[k * nxblock + i] = int((mx + a) / d)
    return first, last


@pytest.mark.parametrize("elem", ["f64", "f32"])
def test_oracle_windows_match_reference_loops(elem):
    rng = np.random.default_rng(7)
    t = rng.uniform(-0.3, 4.0, size=(48, 96))
    for before, after, dt in ((0.1, 0.5, 0.01), (0.0, 0.0, 4e-4), (1.3, 0.07, 0.003)):
        want = reference_slide(t, before, after, dt, elem)
        got = O.punch_windows(t, before, after, dt, elem)
        np.testing.assert_array_equal(got[0], want[0])
        np.testing.assert_array_equal(got[1], want[1])


@pytest.mark.parametrize("elem", ["f64", "f32"])
@pytest.mark.parametrize("nx,nz", [(96, 48), (100, 37), (31, 15), (1, 1)])
def test_product_windows_bit_exact(elem, nx, nz):
    _lib_or_skip()
    rng = np.random.default_rng(nx * 1000 + nz)
    t = rng.uniform(-2.0, 50.0, size=(nz, nx))
    if nx * nz > 20:
        t.flat[3] = np.nan            # skipped by min / max
        t.flat[7] = 1e40 if elem == "f64" else np.inf   # saturates the last step
        t.flat[11] = -1e40 if elem == "f64" else -np.inf
    for before, after, dt in ((0.25, 0.75, 0.01), (0.0, 3.0, 1e-9)):
        want = O.punch_windows(t, before, after, dt, elem)
        got = F.punch_windows(t, before, after, dt, elem)
        np.testing.assert_array_equal(got[0], want[0])
        np.testing.assert_array_equal(got[1], want[1])
    assert F.punch_tiles(nx, nz) == ((nx + 31) // 32, (nz + 15) // 16)


def test_read_punch_file(tmp_path):
    _lib_or_skip()
    nx, nz = 64, 32
    rng = np.random.default_rng(2)
    t = rng.uniform(0.0, 3.0, size=(nz, nx))
    for elem, typ in (("f64", np.float64), ("f32", np.float32)):
        p = tmp_path / ("t_" + elem)
        t.astype(typ).tofile(str(p))
        got = F.read_punch(str(p), nx, nz, 0.2, 0.4, 0.01, elem)
        want = O.punch_windows(t.astype(typ), 0.2, 0.4, 0.01, elem)
        np.testing.assert_array_equal(got[0], want[0])
        np.testing.assert_array_equal(got[1], want[1])
    short = tmp_path / "short"
    t[:10].tofile(str(short))
    with pytest.raises(F.Fd23Error):
        F.read_punch(str(short), nx, nz, 0.2, 0.4, 0.01, "f64")
    with pytest.raises(F.Fd23Error):
        F.read_punch(str(tmp_path / "missing"), nx, nz, 0.2, 0.4, 0.01, "f64")
    out = np.zeros(8, np.int32)
    assert F.lib().fd23_punch_windows(F._p(t), 5, nx, nz, 0.0, 0.0, 0.01, F._p(out), F._p(out)) == F.ERR_ARG


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_oracle_open_windows_equal_plain_run(wave):
    c = Case(wave, 100, 70, npml=10, nt=40, seed=5)
    nb = ((100 + 31) // 32) * ((70 + 15) // 16)
    plain, st = c.oracle("f32")
    w, stw = c.oracle("f32", punch=(np.full(nb, -1, np.int32), np.full(nb, 10 ** 6, np.int32)))
    for a, b in zip(plain, w):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(st, stw)


def test_oracle_closed_windows_keep_state():
    """No tile is ever updated: every wavefield value stays zero except the
    source cells, which sum the source amplitudes step by step."""
    c = Case("psv", 96, 64, npml=10, nt=30, seed=1, kind=3)
    nb = 3 * 4
    _, st = c.oracle("f32", punch=(np.full(nb, 10 ** 6, np.int32), np.full(nb, 10 ** 6, np.int32)))
    field, idx, amp = c.terms
    want = np.zeros(5 * 96 * 64, np.float32)
    for it in range(30):
        for t in range(len(field)):
            if it < amp.shape[1]:
                k = field[t] * 96 * 64 + idx[t]
                want[k] = want[k] + np.float32(amp[t, it])
    np.testing.assert_array_equal(st[:5 * 96 * 64], want)
    assert not np.any(st[5 * 96 * 64:])


def test_oracle_straight_ray_windows_close_to_plain_run():
    """Windows from straight-ray times at the fastest velocity open before
    the first arrival: once the waves have reached every receiver the
    seismograms stay within 1e-6 (relative L2) of the run without windows
    (10 steps of margin); only the stencil's numerical precursor ahead of the
    wavefront is cut, and less of it the earlier the windows open."""
    c = Case("psv", 192, 96, npml=12, nt=400, seed=4, xs=96, zs=20, wavelet=("ricker", 2.0))
    (su, sw), _ = c.oracle("f64")
    errs = []
    for margin in (3, 10, 30):
        first, last = O.punch_windows(c.straight_times(), margin * c.dt, 1e3, c.dt, "f64")
        assert np.any(first > 5)  # some tiles do start late
        (pu, pw), _ = c.oracle("f64", punch=(first, last))
        errs.append(max(O.rel_l2(pu, su), O.rel_l2(pw, sw)))
    assert errs[1] < 1e-6
    assert errs[0] > errs[1] > errs[2]
