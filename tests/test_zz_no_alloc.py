"""The allocation-free watchdog entry point (fd23_sum_squares_noalloc).

Callers that cannot allocate device memory -- code running inside a CUDA
stream capture, programs whose device memory is owned by another allocator --
use this entry point instead of fd23_field_norm2.  This test calls it through
the C ABI on device arrays holding a solver's wavefields and checks it
against fd23_field_norm2 of the same solver, with the tolerance of
test_gpu_parity.py::test_norm2_watchdog (1e-9 relative), on two calls in a
row (its scratch keeps the previous call's contents, which must not leak
into the next result).  The file name sorts last so that a run that stops at
the first failure has already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_sum_squares_matches_solver_norm():
    import torch
    import fd23_gb300 as F
    from tests.fd23_cases import Case
    case = Case("psv", 257, 131, npml=12, nt=40, seed=21)
    s = case.solver("f32")
    s.run(40)
    ref = s.norm2()
    state = s.get_state()
    n = case.nx * case.nz
    fields = [torch.from_numpy(state[k * n:(k + 1) * n].copy()).cuda() for k in range(5)]
    torch.cuda.synchronize()
    ptrs = [t.data_ptr() for t in fields]
    first, bad1 = F.sum_squares_noalloc("f32", ptrs, n)
    # a second call right after; a different input in between would show leftovers
    half, _ = F.sum_squares_noalloc("f32", ptrs[:2], n)
    second, bad2 = F.sum_squares_noalloc("f32", ptrs, n)
    assert not bad1 and not bad2
    assert ref > 0
    assert abs(first - ref) <= 1e-9 * ref
    assert abs(second - ref) <= 1e-9 * ref
    assert half < first
    s.close()


def test_noalloc_rejects_more_fields_than_its_scratch_holds():
    import torch
    import fd23_gb300 as F
    t = torch.ones(16, device="cuda", dtype=torch.float32)
    with pytest.raises(F.Fd23Error) as e:
        F.sum_squares_noalloc("f32", [t.data_ptr()] * 9, 16)
    assert e.value.status == -1
    total, bad = F.sum_squares_noalloc("f32", [t.data_ptr()] * 8, 16)
    assert total == 8 * 16 and not bad
