"""Material table (mktable) on the GPU: on a model with few distinct material
tuples the index + table form gives bit for bit the results of the material
arrays (and of the oracle) for both sweeps, P-SV and SH, every storage form,
with tile step windows and in batches; models with too many tuples are
refused (and a table in use is dropped when the material stops fitting)."""
import numpy as np
import pytest

from oracle import fd23_oracle as O
from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")


def blocky(c, seed):
    """Replace the case's model by flat layers, a dipping interface and a
    rectangular inclusion: a handful of materials, many neighbour patterns."""
    rng = np.random.default_rng(seed)
    nz, nx = c.nz, c.nx
    zz, xx = np.mgrid[0:nz, 0:nx]
    vp = np.full((nz, nx), 3.0)
    for k, depth in enumerate(sorted(rng.integers(nz // 8, nz - 4, size=3))):
        vp[zz >= depth] = 3.5 + 0.6 * k
    vp[zz > nz // 2 + (xx - nx // 2) // 3] += 0.4          # dipping interface
    vp[nz // 4:nz // 4 + 9, nx // 3:nx // 3 + 13] = 5.9     # inclusion
    vs = vp / 1.73
    den = 0.31 * vp ** 0.25 * 8.0
    c.vp, c.vs, c.den = vp, vs, den
    if c.wave == "psv":
        c.mat, c.stab, rc = O.psv_material(vp, vs, den, c.h, c.dt)
    else:
        c.mat, c.stab, rc = O.sh_material(vs, den, c.h, c.dt)
    assert rc == 0
    return c


def expected_entries(c, prec):
    """Distinct storage tuples (+ the zero tuple of the padding)."""
    dt = np.float64 if prec == "f64" else np.float32
    m = np.asarray(c.mat, dt).reshape(c.mat.shape[0], -1).T
    bits = m.view(np.uint64 if dt == np.float64 else np.uint32)  # bit patterns, as the table matches
    rows = np.unique(bits, axis=0)
    return len(rows) + (0 if (rows == 0).all(axis=1).any() else 1)


def _run(c, prec, kernel, table, punch=None, nt=None):
    s = c.solver(prec, kernel)
    n = s.set_material_table(True) if table else None
    if punch is not None:
        s.set_punch(*punch)
    s.run(c.nt if nt is None else nt, 1)
    out = [s.seismograms(f) for f in range(2 if c.wave == "psv" else 1)], s.get_state(), n
    s.close()
    return out


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("kernel", ["fused", "twopass"])
@pytest.mark.parametrize("wave,nx,nz", [("psv", 230, 150), ("psv", 256, 128), ("sh", 230, 150)])
def test_table_parity_with_oracle(wave, nx, nz, kernel, prec):
    c = blocky(Case(wave, nx, nz, npml=12, nt=60, seed=3, topabsorb=int(nx == 256)), seed=nx)
    seis_o, st_o = c.oracle(prec)
    seis, st, n = _run(c, prec, kernel, True)
    assert n == expected_entries(c, prec) and n <= 256
    for a, b in zip(seis, seis_o):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(st, st_o)


@pytest.mark.parametrize("prec", ["bf16", "f16"])
@pytest.mark.parametrize("wave", ["psv", "sh"])
@pytest.mark.parametrize("kernel", ["fused", "twopass"])
def test_table_reduced_storage_equals_arrays(wave, prec, kernel):
    c = blocky(Case(wave, 230, 150, npml=12, nt=60, seed=4), seed=7)
    a, sa, _ = _run(c, prec, kernel, True)
    b, sb, _ = _run(c, prec, kernel, False)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(sa, sb)


def test_table_with_punch_and_batch():
    nt = 50
    cases = [blocky(Case("psv", nx, nz, npml=12, nt=nt, seed=k, xs=nx // 3, zs=nz // 5), seed=k)
             for k, (nx, nz) in enumerate(((230, 150), (400, 123), (161, 310)))]
    rng = np.random.default_rng(2)
    wins = []
    for c in cases:
        nb = ((c.nx + 31) // 32) * ((c.nz + 15) // 16)
        f = rng.integers(-3, nt // 2, size=nb).astype(np.int32)
        wins.append((f, (f + rng.integers(-2, nt, size=nb)).astype(np.int32)))
    # table + windows = oracle with windows
    for c, w in zip(cases, wins):
        seis_o, st_o = c.oracle("f32", punch=w)
        seis, st, _ = _run(c, "f32", "fused", True, punch=w)
        np.testing.assert_array_equal(seis[0], seis_o[0])
        np.testing.assert_array_equal(st, st_o)
    # a batch of tabled shots = the shots alone
    alone = [_run(c, "f32", "fused", True) for c in cases]
    solvers = [c.solver("f32", "fused") for c in cases]
    for s in solvers:
        s.set_material_table(True)
    b = F.Batch(solvers)
    b.run(nt, 1)
    for s, (seis, st, _) in zip(solvers, alone):
        np.testing.assert_array_equal(s.seismograms(1), seis[1])
        np.testing.assert_array_equal(s.get_state(), st)
    b.close()
    solvers[1].set_material_table(False)  # mixed: refused
    b = F.Batch(solvers)
    with pytest.raises(F.Fd23Error) as e:
        b.run(2, 1)
    assert e.value.status == F.ERR_UNSUPPORTED
    b.close()
    for s in solvers:
        s.close()


def test_table_limits():
    c = Case("psv", 160, 96, npml=12, nt=20, seed=1)  # smooth lateral perturbation: every cell differs
    s = c.solver("f32", "fused")
    with pytest.raises(F.Fd23Error) as e:
        s.set_material_table(True)
    assert e.value.status == F.ERR_UNSUPPORTED
    s.run(20, 1)  # the material arrays serve as before
    ref, st_ref = c.oracle("f32")
    np.testing.assert_array_equal(s.get_state(), st_ref)
    s.close()
    # a table in use is rebuilt for a new material, and dropped when it stops fitting
    b = blocky(Case("psv", 160, 96, npml=12, nt=20, seed=1), seed=5)
    s = b.solver("f32", "fused")
    assert s.set_material_table(True) == expected_entries(b, "f32")
    s.set_model(c.vp, c.vs, c.den)  # too many tuples: the table goes, the model stays
    s.run(20, 1)
    np.testing.assert_array_equal(s.get_state(), st_ref)
    s.set_model(b.vp, b.vs, b.den)
    assert s.set_material_table(True) > 1
    with pytest.raises(F.Fd23Error) as e:
        s.set_box(10, 10, 40, 30)
    assert e.value.status == F.ERR_UNSUPPORTED
    s.set_material_table(False)
    s.set_box(10, 10, 40, 30)
    with pytest.raises(F.Fd23Error) as e:
        s.set_material_table(True)
    assert e.value.status == F.ERR_UNSUPPORTED
    s.close()
