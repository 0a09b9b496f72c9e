"""Full-size properties on the GPU: at the 4000 x 2000 size of the benchmark
the fused sweep (with the work plan the autotuner picks, hundreds of CTAs,
multi-item work lists) gives bit for bit the wavefields and seismograms of
the two-pass sweep, one thread per cell, for P-SV and SH; and the oracle's
FP32 run of a 1000 x 500 cut with the benchmark's CPML equals the fused run
bit for bit."""
import numpy as np
import pytest

from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")


def _shot(c, kernel, tune=False, nt=None):
    s = c.solver("f32", kernel)
    if tune:
        s.autotune(5)
    s.run(c.nt if nt is None else nt, 1)
    out = [s.seismograms(f) for f in range(2 if c.wave == "psv" else 1)], s.get_state()
    s.close()
    return out


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_fused_equals_twopass_full_size(wave):
    c = Case(wave, 4000, 2000, npml=40, h=0.005, dt=4e-4, nt=300, seed=11, xs=2000, zs=20,
             wavelet=("ricker", 25.0))
    (sf, stf) = _shot(c, "fused", tune=True)
    (st_, stt) = _shot(c, "twopass")
    for a, b in zip(sf, st_):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(stf, stt)
    assert np.abs(sf[0]).max() > 0


def test_fused_equals_oracle_benchmark_cpml():
    c = Case("psv", 1000, 500, npml=40, h=0.005, dt=4e-4, nt=200, seed=12, xs=500, zs=20,
             wavelet=("ricker", 25.0))
    seis_o, st_o = c.oracle("f32")
    seis, st = _shot(c, "fused", tune=True)
    for a, b in zip(seis, seis_o):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(st, st_o)


@pytest.mark.parametrize("prec", ["f32", "f16"])
def test_banded_plan_keeps_results(prec):
    """The banded work plan (every strip cut on its own) at the benchmark
    size gives bit for bit the strip-major plan's wavefields and seismograms;
    at the 1000 x 500 cut, the oracle's FP32 run."""
    c = Case("psv", 4000, 2000, npml=40, h=0.005, dt=4e-4, nt=120, seed=14, xs=2000, zs=20,
             wavelet=("ricker", 25.0))
    out = {}
    for bands in (0, 1):
        s = c.solver(prec, "fused")
        s.set_plan(5.0, 2.5, 3, 1.0, bands=bands)
        assert s.plan()["bands"] == bands
        s.run(c.nt, 1)
        out[bands] = [s.seismograms(0), s.seismograms(1), s.get_state()]
        s.close()
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)
    if prec == "f32":
        c = Case("psv", 1000, 500, npml=40, h=0.005, dt=4e-4, nt=150, seed=15, xs=500, zs=20,
                 wavelet=("ricker", 25.0))
        seis_o, st_o = c.oracle("f32")
        s = c.solver("f32", "fused")
        s.set_plan(4.0, 3.0, 3, 2.0, bands=1)
        s.run(c.nt, 1)
        np.testing.assert_array_equal(s.seismograms(0), seis_o[0])
        np.testing.assert_array_equal(s.seismograms(1), seis_o[1])
        np.testing.assert_array_equal(s.get_state(), st_o)
        s.close()
