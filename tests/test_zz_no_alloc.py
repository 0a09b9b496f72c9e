"""The allocation-free watchdog entry point (fd23_sum_squares_noalloc).

Programs whose device memory is owned by another allocator (a framework's
caching allocator, a pool sized at start-up) cannot let this library call
cudaMalloc; they use this entry point instead of fd23_field_norm2.  These
tests call it through the C ABI on device arrays holding a solver's
wavefields and check it against fd23_field_norm2 of the same solver, with the
tolerance of test_gpu_parity.py::test_norm2_watchdog (1e-9 relative), on two
calls in a row (its scratch keeps the previous call's contents, which must not
leak into the next result), for every storage type, on the default stream and
on a caller's stream.  The file name sorts last so that a run that stops at
the first failure has already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_TORCH_DTYPE = {"f32": "float32", "f64": "float64", "bf16": "bfloat16", "f16": "float16"}


@pytest.mark.parametrize("prec", ["f32", "f64", "bf16", "f16"])
def test_noalloc_sum_squares_matches_solver_norm(prec):
    import torch
    import fd23_gb300 as F
    from tests.fd23_cases import Case
    case = Case("psv", 257, 131, npml=12, nt=40, seed=21)
    s = case.solver(prec)
    s.run(40)
    ref = s.norm2()
    # the solver's own stored wavefields (buffer set in use, padded layout)
    ptrs = s.field_ptrs()
    n = s.stored_elems()
    first, bad1 = F.sum_squares_noalloc(prec, ptrs, n)
    # a smaller call in between would show leftovers in the shared scratch
    half, _ = F.sum_squares_noalloc(prec, ptrs[:2], n)
    second, bad2 = F.sum_squares_noalloc(prec, ptrs, n)
    assert not bad1 and not bad2
    assert ref > 0
    assert abs(first - ref) <= 1e-9 * ref
    assert abs(second - ref) <= 1e-9 * ref
    assert half < first
    # on a caller's stream (the solver's stream has finished: norm2 waited)
    side = torch.cuda.Stream()
    on_side, bad3 = F.sum_squares_noalloc(prec, ptrs, n, stream=side.cuda_stream)
    assert not bad3 and abs(on_side - ref) <= 1e-9 * ref
    s.close()


@pytest.mark.parametrize("prec", ["f32", "f64", "bf16", "f16"])
def test_noalloc_flags_nan_and_inf(prec):
    import torch
    import fd23_gb300 as F
    dt = getattr(torch, _TORCH_DTYPE[prec])
    a = torch.full((1000,), 0.5, dtype=dt, device="cuda")
    b = torch.full((1000,), 0.25, dtype=dt, device="cuda")
    total, bad = F.sum_squares_noalloc(prec, [a.data_ptr(), b.data_ptr()], 1000)
    assert not bad and total == pytest.approx(1000 * (0.25 + 0.0625), rel=1e-12)
    a[17] = float("nan")
    _, bad = F.sum_squares_noalloc(prec, [a.data_ptr(), b.data_ptr()], 1000)
    assert bad
    a[17] = 0.5
    b[999] = float("inf")
    _, bad = F.sum_squares_noalloc(prec, [a.data_ptr(), b.data_ptr()], 1000)
    assert bad
    b[999] = 0.25
    total, bad = F.sum_squares_noalloc(prec, [a.data_ptr(), b.data_ptr()], 1000)
    assert not bad and total == pytest.approx(1000 * (0.25 + 0.0625), rel=1e-12)


def test_noalloc_rejects_more_fields_than_its_scratch_holds():
    import torch
    import fd23_gb300 as F
    t = torch.ones(16, device="cuda", dtype=torch.float32)
    with pytest.raises(F.Fd23Error) as e:
        F.sum_squares_noalloc("f32", [t.data_ptr()] * 9, 16)
    assert e.value.status == -1
    total, bad = F.sum_squares_noalloc("f32", [t.data_ptr()] * 8, 16)
    assert total == 8 * 16 and not bad


def test_noalloc_rejects_host_memory():
    import numpy as np
    import fd23_gb300 as F
    h = np.ones(16, dtype=np.float32)
    with pytest.raises(F.Fd23Error) as e:
        F.sum_squares_noalloc("f32", [h.ctypes.data], 16)
    assert e.value.status == -1


def test_noalloc_declines_a_capturing_stream_and_leaves_the_capture_valid():
    import torch
    import fd23_gb300 as F
    x = torch.zeros(64, device="cuda")
    y = torch.ones(64, device="cuda")
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    status = None
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            x.add_(1.0)
            try:
                F.sum_squares_noalloc("f32", [y.data_ptr()], 64, stream=side.cuda_stream)
            except F.Fd23Error as e:
                status = e.status
            x.add_(1.0)
    assert status == F.ERR_UNSUPPORTED
    g.replay()
    torch.cuda.synchronize()
    assert torch.all(x == 2.0)
    total, bad = F.sum_squares_noalloc("f32", [y.data_ptr()], 64)
    assert total == 64.0 and not bad
