"""Batched shots and the work-plan autotuner on the GPU: a batch of uneven
shots advanced in lockstep (one sweep launch per step, CUDA-graph captured)
gives every shot exactly the seismograms and state it gets alone; split runs,
graph replay and direct launches agree; autotuning changes only the schedule."""
import numpy as np
import pytest

from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")

# uneven grids (none a tile multiple), different sources, models and CPML tops
SHOTS = [
    dict(nx=230, nz=150, seed=1, kind=3, topabsorb=0),
    dict(nx=97, nz=70, seed=2, kind=13, topabsorb=1),
    dict(nx=400, nz=123, seed=3, kind=1, topabsorb=0),
    dict(nx=161, nz=310, seed=4, kind=3, topabsorb=0),
    dict(nx=1013, nz=517, seed=5, kind=3, topabsorb=0),
]


def _cases(wave, nt):
    out = []
    for d in SHOTS:
        kind = d["kind"]
        if wave == "sh":
            kind = {1: 2, 13: 13, 3: 3}[kind]
        out.append(Case(wave, d["nx"], d["nz"], npml=12, nt=nt, seed=d["seed"], kind=kind,
                        topabsorb=d["topabsorb"]))
    return out


def _run_alone(cases, prec, nt, itrecord=1):
    res = []
    for c in cases:
        s = c.solver(prec, "fused")
        s.run(nt, itrecord)
        res.append(([s.seismograms(f) for f in range(2 if c.wave == "psv" else 1)], s.get_state()))
        s.close()
    return res


@pytest.mark.parametrize("wave,prec", [("psv", "f32"), ("psv", "f64"), ("psv", "bf16"), ("sh", "f32"),
                                       ("sh", "f16")])
def test_batch_equals_shots_alone(wave, prec):
    nt = 50
    cases = _cases(wave, nt)
    alone = _run_alone(cases, prec, nt, itrecord=2)
    solvers = [c.solver(prec, "fused") for c in cases]
    b = F.Batch(solvers)
    assert b.plan()["nblocks"] >= len(cases)
    b.run(nt, 2)
    for s, (seis, st) in zip(solvers, alone):
        assert s.step == nt
        for f, ref in enumerate(seis):
            np.testing.assert_array_equal(s.seismograms(f), ref)
        np.testing.assert_array_equal(s.get_state(), st)
    b.close()
    for s in solvers:
        s.close()


def test_batch_split_replay_and_direct_launches():
    nt = 40
    cases = _cases("psv", nt)
    alone = _run_alone(cases, "f32", nt)
    solvers = [c.solver("f32", "fused") for c in cases]
    b = F.Batch(solvers)
    b.run(15, 1)  # captured graph
    b.run(25, 1)
    for s, (seis, st) in zip(solvers, alone):
        np.testing.assert_array_equal(s.seismograms(0), seis[0])
        np.testing.assert_array_equal(s.get_state(), st)
    # same step range again: the cached graph is replayed
    for s in solvers:
        s.reset()
    b.run(15, 1)
    b.run(25, 1)
    b.sync()
    for s, (seis, st) in zip(solvers, alone):
        np.testing.assert_array_equal(s.seismograms(1), seis[1])
        np.testing.assert_array_equal(s.get_state(), st)
    # step-by-step launches
    b.set_graph(False)
    for s in solvers:
        s.reset()
    b.run(nt, 1)
    for s, (seis, st) in zip(solvers, alone):
        np.testing.assert_array_equal(s.get_state(), st)
    b.close()
    for s in solvers:
        s.close()


def test_autotune_keeps_results():
    nt = 60
    c = Case("psv", 700, 380, npml=20, nt=nt, seed=8)
    ref = c.solver("f32", "fused")
    ref.run(nt, 1)
    s = c.solver("f32", "fused")
    s.run(20, 1)
    trials = s.autotune(3)
    assert len(trials) >= 8 and all(t["ms_per_step"] > 0 for t in trials)
    assert s.step == 20
    s.run(nt - 20, 1)
    np.testing.assert_array_equal(s.seismograms(0), ref.seismograms(0))
    np.testing.assert_array_equal(s.get_state(), ref.get_state())
    # the same through a batch
    cases = _cases("psv", nt)
    alone = _run_alone(cases, "f32", nt)
    solvers = [x.solver("f32", "fused") for x in cases]
    b = F.Batch(solvers)
    b.run(10, 1)
    bt = b.autotune(3)
    assert len(bt) >= 8
    b.run(nt - 10, 1)
    for x, (seis, st) in zip(solvers, alone):
        np.testing.assert_array_equal(x.seismograms(0), seis[0])
        np.testing.assert_array_equal(x.get_state(), st)
    b.close()
    for x in solvers + [s, ref]:
        x.close()


def test_batch_errors():
    cases = _cases("psv", 10)[:2]
    a, c = cases[0].solver("f32", "fused"), cases[1].solver("f32", "fused")
    a.run(1, 1)
    b = F.Batch([a, c])
    with pytest.raises(F.Fd23Error) as e:
        b.run(2, 1)  # not in lockstep
    assert e.value.status == F.ERR_ORDER
    b.close()
    d = cases[1].solver("bf16", "fused")
    with pytest.raises(F.Fd23Error):
        F.Batch([a, d])  # mixed precision
    t = cases[1].solver("f32", "twopass")
    with pytest.raises(F.Fd23Error) as e:
        F.Batch([a, t])
    assert e.value.status == F.ERR_UNSUPPORTED
    with pytest.raises(F.Fd23Error):
        F.Batch([a, a])
    for x in (a, c, d, t):
        x.close()
