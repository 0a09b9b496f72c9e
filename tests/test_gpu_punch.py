"""usepunch (tile step windows) on the GPU: bit-exact parity with the
oracle's windowed run for both sweeps, P-SV and SH, FP32 and FP64, under
random windows that open and close (source tiles included); 16-bit forms
fused = two-pass; batches, split runs, restarts and the autotuner keep the
results; the windows skip work without changing the physics of a run whose
windows open before the first arrival."""
import numpy as np
import pytest

from oracle import fd23_oracle as O
from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")


def random_windows(nx, nz, seed, nt):
    """Windows that open and close at random steps: never open, always open,
    short and long; about a third of the tiles are left alone at any step."""
    rng = np.random.default_rng(seed)
    nb = ((nx + 31) // 32) * ((nz + 15) // 16)
    first = rng.integers(-3, nt // 2, size=nb)
    last = first + rng.integers(-2, nt, size=nb)
    k = rng.permutation(nb)
    first[k[:nb // 8]], last[k[:nb // 8]] = -1, 10 ** 6            # always updated
    first[k[nb // 8:nb // 4]], last[k[nb // 8:nb // 4]] = 10 ** 6, 10 ** 6  # never
    return first.astype(np.int32), last.astype(np.int32)


def _run(c, prec, kernel, punch, nt=None, phase=None):
    nt = c.nt if nt is None else nt
    s = c.solver(prec, kernel)
    if punch is not None:
        s.set_punch(*punch)
    if phase is not None:
        s.set_punch_phase(phase)
    s.run(nt, 1)
    out = [s.seismograms(f) for f in range(2 if c.wave == "psv" else 1)], s.get_state()
    s.close()
    return out


CASES = [
    # wave, nx, nz, kind, topabsorb
    ("psv", 256, 160, 3, 0),
    ("psv", 230, 150, 13, 1),
    ("sh", 256, 160, 3, 0),
    ("sh", 230, 150, 2, 0),
]


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("kernel", ["fused", "twopass"])
@pytest.mark.parametrize("wave,nx,nz,kind,topabsorb", CASES)
def test_punch_parity_with_oracle(wave, nx, nz, kind, topabsorb, prec, kernel):
    nt = 60
    c = Case(wave, nx, nz, npml=12, nt=nt, seed=nx + kind, kind=kind, topabsorb=topabsorb,
             xs=nx // 2 + 3, zs=nz // 4 + 5)
    w = random_windows(nx, nz, seed=nx * 7 + kind, nt=nt)
    seis_o, st_o = c.oracle(prec, punch=w)
    # phase plans of 7 steps (several rebuilds, buffer reuse), and the static plan
    for phase in ((7, 0) if kernel == "fused" else (None,)):
        seis, st = _run(c, prec, kernel, w, phase=phase)
        for a, b in zip(seis, seis_o):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(st, st_o)
    # the windows did change the run
    plain, _ = c.oracle(prec)
    assert not np.array_equal(plain[0], seis_o[0])


@pytest.mark.parametrize("prec", ["bf16", "f16"])
@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_punch_reduced_storage_fused_equals_twopass(prec, wave):
    c = Case(wave, 230, 150, npml=12, nt=60, seed=3)
    w = random_windows(230, 150, seed=11, nt=60)
    a, sa = _run(c, prec, "fused", w)
    b, sb = _run(c, prec, "twopass", w)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(sa, sb)


def test_punch_batch_equals_shots_alone():
    nt = 50
    cases = [Case("psv", nx, nz, npml=12, nt=nt, seed=s, xs=nx // 3, zs=nz // 5)
             for nx, nz, s in ((230, 150, 1), (400, 123, 2), (161, 310, 3), (300, 200, 4))]
    wins = [random_windows(c.nx, c.nz, seed=k + 40, nt=nt) for k, c in enumerate(cases)]
    wins[3] = None  # one shot without windows
    alone = [_run(c, "f32", "fused", w) for c, w in zip(cases, wins)]
    solvers = []
    for c, w in zip(cases, wins):
        s = c.solver("f32", "fused")
        if w is not None:
            s.set_punch(*w)
        solvers.append(s)
    b = F.Batch(solvers)
    b.run(20, 1)
    b.run(nt - 20, 1)
    for s, (seis, st) in zip(solvers, alone):
        np.testing.assert_array_equal(s.seismograms(0), seis[0])
        np.testing.assert_array_equal(s.seismograms(1), seis[1])
        np.testing.assert_array_equal(s.get_state(), st)
    b.close()
    for s in solvers:
        s.close()


def test_punch_split_restart_and_autotune():
    """run(a) + autotune + run(b) and a restart from the state at step a,
    with the windows installed afterwards, both equal one run of a+b steps."""
    nt, a = 60, 25
    c = Case("psv", 700, 380, npml=20, nt=nt, seed=8, xs=350, zs=60)
    w = random_windows(700, 380, seed=5, nt=nt)
    ref, st_ref = _run(c, "f32", "fused", w)
    s = c.solver("f32", "fused")
    s.set_punch(*w)
    s.run(a, 1)
    mid = s.get_state()
    assert len(s.autotune(3)) >= 8
    s.run(nt - a, 1)
    np.testing.assert_array_equal(s.seismograms(0), ref[0])
    np.testing.assert_array_equal(s.get_state(), st_ref)
    s.close()
    r = c.solver("f32", "fused")
    r.set_state(mid, a)
    r.set_punch(*w)
    r.run(nt - a, 1)
    np.testing.assert_array_equal(r.seismograms(1), ref[1][a:])
    np.testing.assert_array_equal(r.get_state(), st_ref)
    # windows removed: the plain sweep again, from the same state
    r.set_punch(None, None)
    r.run(2, 1)
    r.close()


def test_punch_errors():
    c = Case("psv", 120, 90, npml=10, nt=10)
    s = c.solver("f32", "fused")
    w = random_windows(120, 90, seed=1, nt=10)
    with pytest.raises(F.Fd23Error) as e:
        s.set_punch(w[0][:-1], w[1][:-1])  # wrong tile count
    assert e.value.status == F.ERR_ARG
    s.set_punch(*w)
    with pytest.raises(F.Fd23Error) as e:
        s.set_box(10, 10, 40, 30)
    assert e.value.status == F.ERR_UNSUPPORTED
    s.set_punch(None, None)
    s.set_box(10, 10, 40, 30)
    with pytest.raises(F.Fd23Error) as e:
        s.set_punch(*w)
    assert e.value.status == F.ERR_UNSUPPORTED
    s.close()


def test_punch_straight_ray_windows_full_size():
    """A 2000 x 1000 shot with windows from straight-ray times (opening 20
    steps early, never closing): the fused sweep skips the quiet tiles, and
    the seismograms stay within 1e-5 of the run without windows (FP32)."""
    nt = 1500
    c = Case("psv", 2000, 1000, npml=30, h=0.005, dt=4e-4, nt=nt, seed=12, xs=1000, zs=20,
             wavelet=("ricker", 15.0))  # km and km/s: at most 0.48 cells per step
    first, last = O.punch_windows(c.straight_times(), 20 * c.dt, 1e3, c.dt, "f64")
    assert (first > nt).mean() > 0.3  # a good part of the grid stays quiet throughout
    plain, _ = _run(c, "f32", "fused", None)
    win, _ = _run(c, "f32", "fused", (first, last))
    for a, b in zip(win, plain):
        assert O.rel_l2(a, b) < 1e-5
