"""The persistent form (FD23_KERNEL_PERSIST): a whole run in one cooperative
launch of the two-pass updates with grid barriers between the phases.  Its
wavefields, memory variables and seismograms equal the two-pass sweep's bit
for bit (and the oracle's for FP32 / FP64) over P-SV and SH, every storage
form, every source kind, stress receivers, record decimation, split runs,
tile step windows, the material table, an absorbing top and a fluid layer;
a persistent solver with a hybrid box steps like the two-pass sweep."""
import numpy as np
import pytest

from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")


def _run(c, prec, kernel, nt=None, itrecord=1, split=None, stress_rec=False, punch=None, table=False):
    s = c.solver(prec, kernel)
    if table:
        s.set_material_table(True)
    if punch is not None:
        s.set_punch(*punch)
    if stress_rec:
        s.set_receivers(2 if c.wave == "psv" else 1, c.rx[:5], c.rz[:5] + 3)
    nt = c.nt if nt is None else nt
    if split:
        s.run(split, itrecord)
        s.run(nt - split, itrecord)
    else:
        s.run(nt, itrecord)
    nf = 5 if c.wave == "psv" else 3
    out = [s.seismograms(f) for f in range(nf) if s.seismograms(f).size], s.get_state()
    s.close()
    return out


def _same(a, b):
    for x, y in zip(a[0], b[0]):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("prec", ["f32", "f64", "bf16", "f16"])
@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_persist_equals_twopass(wave, prec):
    c = Case(wave, 230, 150, npml=12, nt=70, seed=3, topabsorb=1)
    _same(_run(c, prec, "persist"), _run(c, prec, "twopass"))


@pytest.mark.parametrize("wave,kind", [("psv", 3), ("psv", 13), ("psv", 1), ("sh", 3), ("sh", 13), ("sh", 2)])
def test_persist_sources_and_oracle(wave, kind):
    c = Case(wave, 181, 97, npml=10, nt=60, seed=5, kind=kind, xs=90, zs=1 if kind != 1 else 30)
    got = _run(c, "f32", "persist")
    seis_o, st_o = c.oracle("f32")
    for a, b in zip(got[0], seis_o):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(got[1], st_o)


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_persist_receivers_splits_decimation(wave):
    c = Case(wave, 200, 120, npml=12, nt=61, seed=8, fluid=wave == "psv")
    ref = _run(c, "f64", "twopass", itrecord=3, stress_rec=True)
    _same(_run(c, "f64", "persist", itrecord=3, stress_rec=True), ref)
    _same(_run(c, "f64", "persist", itrecord=3, stress_rec=True, split=25), ref)
    _same(_run(c, "f32", "persist", itrecord=2), _run(c, "f32", "twopass", itrecord=2))


def test_persist_punch_and_table():
    c = Case("psv", 300, 140, npml=12, nt=50, seed=2, xs=150, zs=30)
    nb = ((c.nx + 31) // 32) * ((c.nz + 15) // 16)
    rng = np.random.default_rng(1)
    first = rng.integers(-3, 25, size=nb).astype(np.int32)
    last = (first + rng.integers(-2, 50, size=nb)).astype(np.int32)
    _same(_run(c, "f32", "persist", punch=(first, last)), _run(c, "f32", "twopass", punch=(first, last)))
    vp = np.full((c.nz, c.nx), 4.0)
    vp[c.nz // 2:] = 5.0
    c.vp, c.vs, c.den = vp, vp / 1.73, 0.31 * vp ** 0.25 * 8.0
    _same(_run(c, "f32", "persist", table=True), _run(c, "f32", "twopass", table=True))


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_persist_larger_grids(wave):
    """More cells than threads in flight (several cells per thread and phase)."""
    c = Case(wave, 1500, 700, npml=20, nt=30, seed=4, xs=700, zs=40)
    _same(_run(c, "f32", "persist"), _run(c, "f32", "twopass"))


def test_persist_box_steps_like_twopass():
    from tests.test_gpu_line_source import _box_setup
    c, mat, bmat, box, desc, src, inc = _box_setup("f32", nt=40)
    outs = []
    for kernel in ("persist", "twopass"):
        s = F.Solver("psv", c.nx, c.nz, c.npml, c.h, c.dt, prec="f32", kernel=kernel, **c.pml)
        s.set_material(mat)
        s.set_receivers(0, c.rx, c.rz)
        s.set_box(*box, bmat=bmat)
        s.set_box_line_source(desc, src, bmat, 0, 40)
        s.run(40, 1)
        outs.append((s.seismograms(0), s.get_state()))
        s.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])
    s = Case("psv", 100, 80, npml=8, nt=5).solver("f32", "persist")
    with pytest.raises(F.Fd23Error) as e:  # batches take fused solvers only
        F.Batch([s])
    assert e.value.status == F.ERR_UNSUPPORTED
    s.close()
