"""Strips whose origin lies left of column 0 (the planner moves it there when
that puts the x-CPML into fewer strips; copies left of the array read zeros,
lanes left of column 0 store nothing): grids whose planned origin is -48,
-32 and -24 give bit for bit the oracle's results (P-SV and SH, FP32 and
FP64), the two-pass sweep's (16-bit storage, the hybrid box) and the
material-table form's, alone and in a batch."""
import numpy as np
import pytest

from oracle import fd23_oracle as O
from tests.fd23_cases import Case
from tests.test_gpu_table import blocky

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")

# (nx, npml) -> planned strip origin, checked below
GRIDS = {(242, 40): -48, (242, 24): -32, (242, 16): -24}


def _origin(nx, nz, npml):
    return min(it[1] for cta in F.work_plan([(nx, nz, npml, 0)]) for it in cta)


def _run(c, prec, kernel, table=False):
    s = c.solver(prec, kernel)
    if table:
        s.set_material_table(True)
    s.run(c.nt, 1)
    out = [s.seismograms(f) for f in range(2 if c.wave == "psv" else 1)], s.get_state()
    s.close()
    return out


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("wave", ["psv", "sh"])
@pytest.mark.parametrize("nx,npml", sorted(GRIDS))
def test_shifted_origin_bit_exact_vs_oracle(nx, npml, wave, prec):
    c = Case(wave, nx, 120, npml=npml, nt=60, seed=nx + npml, xs=npml // 2 + 2, zs=9)
    assert _origin(nx, 120, npml) == GRIDS[(nx, npml)]
    seis_o, st_o = c.oracle(prec)
    seis, st = _run(c, prec, "fused")
    for a, b in zip(seis, seis_o):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(st, st_o)


@pytest.mark.parametrize("prec", ["f16", "bf16"])
@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_shifted_origin_16bit_equals_twopass(wave, prec):
    c = Case(wave, 242, 120, npml=40, nt=60, seed=5, xs=12, zs=9)
    a, sa = _run(c, prec, "fused")
    b, sb = _run(c, prec, "twopass")
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(sa, sb)


def test_shifted_origin_material_table():
    c = blocky(Case("psv", 242, 120, npml=24, nt=60, seed=6, xs=14, zs=9), seed=3)
    seis_o, st_o = c.oracle("f32")
    seis, st = _run(c, "f32", "fused", table=True)
    for a, b in zip(seis, seis_o):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(st, st_o)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_shifted_origin_hybrid_box(prec):
    """a box next to the left CPML (its rings in the first strip) and the
    residual field driven by another run's ring history: fused = two-pass"""
    nx, nz, npml, nt = 242, 120, 16, 50
    box = (20, 30, 40, 36)
    c = Case("psv", nx, nz, npml=npml, nt=nt, xs=120, zs=10, seed=8)
    ci = Case("psv", nx, nz, npml=npml, nt=nt, xs=40, zs=48, seed=22)
    inc, _ = O.psv_ring_history("f64", nx, nz, npml, 0, ci.mat, ci.bck, ci.terms, nt, box)
    inc = inc.astype(np.float64 if prec == "f64" else np.float32)
    out = {}
    for kernel in ("fused", "twopass"):
        s = c.solver(prec, kernel)
        for f in range(5):
            s.set_receivers(f, np.array([21, 25, 59, 100], np.int32), np.array([30, 40, 65, 5], np.int32))
        s.set_box(*box)
        s.set_box_incident(inc, 0)
        s.run(nt, 1)
        out[kernel] = [s.seismograms(f) for f in range(5)] + [s.get_state(), s.get_box_state()]
        s.close()
    assert np.abs(out["fused"][-1]).max() > 0
    for a, b in zip(out["fused"], out["twopass"]):
        np.testing.assert_array_equal(a, b)


def test_shifted_origin_batch():
    """a batch of shots with origins -48, -32, -24 and 0 equals the shots
    run with the two-pass sweep"""
    cases = [Case("psv", nx, 120, npml=npml, nt=40, seed=k, xs=npml // 2 + 2, zs=9)
             for k, (nx, npml) in enumerate(sorted(GRIDS) + [(200, 10)])]
    alone = [_run(c, "f32", "twopass") for c in cases]
    solvers = [c.solver("f32", "fused") for c in cases]
    b = F.Batch(solvers)
    b.set_plan(4.0, 3.0, 3, 3.0, bands=1)
    b.run(40, 1)
    for s, (seis, st) in zip(solvers, alone):
        np.testing.assert_array_equal(s.seismograms(0), seis[0])
        np.testing.assert_array_equal(s.seismograms(1), seis[1])
        np.testing.assert_array_equal(s.get_state(), st)
    b.close()
    for s in solvers:
        s.close()
