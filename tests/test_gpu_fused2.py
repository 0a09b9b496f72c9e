"""GPU parity of the two-step fused sweep (kernel "fused2": two time steps per
launch, every wavefield read and written once per two steps).

Its arithmetic is the one-step sweep's operation sequence, so FP32 results
must equal the CPU oracle (and the one-step sweep) bit for bit: seismograms
of every step (the step in between is recorded inside the launch), the full
state (wavefields and every memory variable), over grids that are not tile
multiples, free-surface and absorbing tops, every P-SV source kind, the
fluid-layer edge rules, odd step counts (the last step runs the one-step
sweep), record decimation, split runs, restarts and stress receivers, for
both strip widths.
"""
import numpy as np
import pytest

from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[256, 128], autouse=True)
def width(request, monkeypatch):
    """both strip widths of the sweep: 256 columns (one CTA per SM) and 128
    (two); read when a solver is created"""
    monkeypatch.setenv("FD23_FUSED2_WIDTH", str(request.param))
    return request.param

PSV_CASES = [
    dict(nx=96, nz=64, kind=3),
    dict(nx=250, nz=130, kind=3, topabsorb=1),
    dict(nx=257, nz=131, kind=13, npml=16),
    dict(nx=300, nz=200, kind=1, fluid=True),
    dict(nx=130, nz=97, kind=3, zs=1, xs=5),  # source next to the surface and the edge
    dict(nx=700, nz=90, kind=3, xs=463, zs=40),  # source on a strip boundary (232-column strips)
    dict(nx=420, nz=77, kind=3, xs=207, zs=30),  # source on a strip boundary (104-column strips)
]


def _run(case, kernel, nt, itrecord=1):
    s = case.solver("f32", kernel)
    s.run(nt, itrecord)
    out = [s.seismograms(0), s.seismograms(1)]
    st = s.get_state()
    s.close()
    return out, st


@pytest.mark.parametrize("nt", [70, 71])
@pytest.mark.parametrize("cfg", PSV_CASES, ids=lambda c: "%dx%d_k%d" % (c["nx"], c["nz"], c["kind"]))
def test_fused2_bit_exact_vs_oracle(cfg, nt):
    case = Case("psv", nt=nt, **cfg)
    ref, ref_state = case.oracle("f32")
    got, state = _run(case, "fused2", nt)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)
    np.testing.assert_array_equal(state, ref_state)


def test_fused2_multi_item_worklist():
    """1000x1000: several 232-column strips cut into row ranges, CTAs owning
    pieces of two strips."""
    case = Case("psv", 1000, 1000, npml=20, nt=40, seed=3)
    ref, ref_state = case.oracle("f32")
    got, state = _run(case, "fused2", 40)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)
    np.testing.assert_array_equal(state, ref_state)


def test_fused2_itrecord_and_split_runs():
    """records every 3rd step (the recorded step falls on either step of a
    launch); runs of odd and even lengths equal one run."""
    case = Case("psv", 200, 120, nt=50, seed=5)
    ref, ref_state = case.oracle("f32", itrecord=3)
    s = case.solver("f32", "fused2")
    s.run(17, 3)
    s.run(20, 3)
    s.run(13, 3)
    np.testing.assert_array_equal(s.seismograms(0), ref[0])
    np.testing.assert_array_equal(s.seismograms(1), ref[1])
    np.testing.assert_array_equal(s.get_state(), ref_state)
    assert s.step == 50
    s.close()


def test_fused2_restart():
    case = Case("psv", 180, 140, nt=60, seed=7, topabsorb=1)
    _, full_state = case.oracle("f32", nt=60)
    a = case.solver("f32", "fused2")
    a.run(25)
    st = a.get_state()
    a.close()
    b = case.solver("f32", "fused2")
    b.set_state(st, 25)
    b.run(35)
    np.testing.assert_array_equal(b.get_state(), full_state)
    b.close()


def test_fused2_stress_receivers_match_one_step_sweep():
    """receivers on all five wavefields, at the surface, on strip edges and
    buried: the two-step sweep records what the one-step sweep records."""
    case = Case("psv", 600, 300, npml=20, nt=44, seed=11)
    rx = np.array([0, 1, 231, 232, 233, 463, 464, 599, 300, 301, 10, 590], dtype=np.int32)
    rz = np.array([0, 0, 0, 0, 5, 150, 151, 299, 3, 4, 290, 7], dtype=np.int32)
    out = {}
    for kernel in ("fused", "fused2"):
        s = case.solver("f32", kernel)
        for f in range(5):
            s.set_receivers(f, rx, rz)
        s.run(44)
        out[kernel] = [s.seismograms(f) for f in range(5)] + [s.get_state()]
        s.close()
    for a, b in zip(out["fused"], out["fused2"]):
        np.testing.assert_array_equal(a, b)


def test_fused2_large_grid_matches_one_step_sweep():
    """2000x1000 with a 40-cell CPML (many items per strip, x-CPML strips
    inside the first and last strips): state after 24 steps equals the
    one-step sweep's bit for bit."""
    case = Case("psv", 2000, 1000, npml=40, nt=24, seed=13)
    st = {}
    for kernel in ("fused", "fused2"):
        s = case.solver("f32", kernel)
        s.run(24)
        st[kernel] = (s.get_state(), s.seismograms(0), s.seismograms(1))
        s.close()
    for a, b in zip(st["fused"], st["fused2"]):
        np.testing.assert_array_equal(a, b)
