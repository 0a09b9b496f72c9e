"""Failure handling on the GPU without a fault: a bounded device-side wait
that runs out (on a barrier nothing completes) raises the solver's error
flag; the host sees FD23_ERR_TIMEOUT, the sweeps stand down, and a reset
makes the solver usable again with unchanged results."""
import numpy as np
import pytest

from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")


def test_wait_that_runs_out_is_reported_and_recoverable():
    c = Case("psv", 140, 100, npml=12, nt=40, seed=6)
    ref = c.solver("f32", "fused")
    ref.run(40, 1)
    want = ref.seismograms(0)
    s = c.solver("f32", "fused")
    s.run(10, 1)
    s.sync()
    F._check(F.lib().fd23_debug_expire_wait(s._h), "fd23_debug_expire_wait")
    with pytest.raises(F.Fd23Error) as e:
        s.sync()
    assert e.value.status == F.ERR_TIMEOUT
    s.run(5, 1)  # sweeps see the flag and return without touching the fields
    with pytest.raises(F.Fd23Error) as e:
        s.sync()
    assert e.value.status == F.ERR_TIMEOUT
    s.reset()
    s.run(40, 1)
    np.testing.assert_array_equal(s.seismograms(0), want)
    s.close()
    ref.close()


@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_persistent_barrier_that_runs_out_is_reported_and_recoverable(wave):
    """The persistent form's grid barrier, made unreachable (one arrival more
    than the launch has), gives up after its bounded wait: the host sees
    FD23_ERR_TIMEOUT, later runs stand down without touching the fields, and
    a reset makes the solver usable again with unchanged results."""
    c = Case(wave, 200, 120, npml=12, nt=40, seed=6)
    ref = c.solver("f32", "persist")
    ref.run(40, 1)
    want = ref.seismograms(0)
    s = c.solver("f32", "persist")
    s.run(10, 1)
    s.sync()
    F._check(F.lib().fd23_debug_persist_barrier(s._h), "fd23_debug_persist_barrier")
    with pytest.raises(F.Fd23Error) as e:
        s.sync()
    assert e.value.status == F.ERR_TIMEOUT
    s.run(5, 1)
    with pytest.raises(F.Fd23Error) as e:
        s.sync()
    assert e.value.status == F.ERR_TIMEOUT
    s.reset()
    s.run(40, 1)
    np.testing.assert_array_equal(s.seismograms(0), want)
    s.close()
    ref.close()
    # a fused solver has no such barrier
    f = c.solver("f32", "fused")
    with pytest.raises(F.Fd23Error) as e:
        F._check(F.lib().fd23_debug_persist_barrier(f._h), "fd23_debug_persist_barrier")
    assert e.value.status == F.ERR_ORDER
    f.close()
