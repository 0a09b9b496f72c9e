"""CPU audit of every address the fused sweep forms (fd23_gb300/csrc/fd23_fused.cu).

Takes the work plans from the library (fd23_work_plan: the planner the
solver and the batch use), restates the padded layout (make_layout) and the
index arithmetic of the kernel, then checks, for the grid sizes the tests and
the benchmarks use (and the 64-shot batch), that

  * every bulk copy reads inside its HBM buffer, starts on a 16-byte boundary
    in global and shared memory, and moves a multiple of 16 bytes;
  * every shared-memory read and write stays inside its ring;
  * every HBM store lands on a cell of the grid;
  * no CTA holds more work items than its item table.

Index expressions are affine in the lane chunk q and the row group g, so the
extreme values q in {0, 31}, g in {0, 3} bound every thread.
"""
import pytest

XPAD = ZPAD = 8
TX, SW = 120, 128
UWW = SW + 8
NUW, NPW, NTR = 4, 2, 4
MAX_ITEMS = 4


def layout(nx, nz):
    ntx = (nx + TX - 1) // TX
    cover_x, cover_z = ntx * TX, (nz + 3) // 4 * 4
    pitch = (XPAD + max(cover_x, nx) + 8 + 31) // 32 * 32
    rows = ZPAD + max(cover_z, nz) + 8
    return pitch, rows, ZPAD * pitch + XPAD


def worklist(nx, nz, npml, oversub=1.0, per_sm=3):
    F = pytest.importorskip("fd23_gb300")
    try:
        F.lib()
    except ImportError as e:
        pytest.skip(str(e))
    return [[it[1:] for it in cta] for cta in F.work_plan([(nx, nz, npml, 0)], per_sm=per_sm, oversub=oversub)]


def audit(nx, nz, es, wave, per_sm=3, oversub=1.0, ctas=None):
    pitch, rows, origin = layout(nx, nz)
    npml = min(40, nx // 2, nz // 2)
    elems = pitch * rows
    nv = 2 if wave == "psv" else 1
    nt = 3 if wave == "psv" else 2
    npf = 8 if wave == "psv" else 5
    pwoff = 4 if es == 2 else 0
    pww = SW + 2 * pwoff
    assert (pitch * es) % 16 == 0
    if ctas is None:
        ctas = worklist(nx, nz, npml, oversub, per_sm)
    covered = set()
    for items in ctas:
        assert 1 <= len(items) <= MAX_ITEMS
        for (x0, z0, z1) in items:
            for zb in range(z0 // 4, z1 // 4):
                key = (x0, zb)
                assert key not in covered  # every block exactly once
                covered.add(key)
        for (x0, z0, z1) in items:
            assert x0 % TX == 0 and z0 % 4 == 0 and z1 % 4 == 0 and z1 > z0
            niter = (z1 - z0) // 4 + 2
            # stencil-input copies: blocks 0 .. niter+1, rows z0-8+4b .. +3
            for b in (0, niter + 1):
                for rr in (0, 3):
                    r = z0 - 8 + 4 * b + rr
                    off = origin + r * pitch + (x0 - 8)
                    assert 0 <= off and off + UWW <= elems, (nx, nz, x0, r)
                    assert (off * es) % 16 == 0 and (UWW * es) % 16 == 0
            # point-wise copies of iterations 0 .. niter-1
            for i in (0, niter - 1):
                for rr in (0, 3):
                    for r in (z0 - 4 + 4 * i + rr, z0 - 8 + 4 * i + rr):
                        off = origin + r * pitch + (x0 - 4 - pwoff)
                        assert 0 <= off and off + pww <= elems
                        assert (off * es) % 16 == 0 and (pww * es) % 16 == 0
            for i in range(niter):
                for g in (0, 3):
                    for q in (0, 31):
                        # stress phase: stencil rows j-4 .. j+4, columns 4q .. 4q+11
                        j = z0 - 4 + 4 * i + g
                        for r in (j - 4, j + 4):
                            blk = (r - (z0 - 8)) // 4
                            assert i <= blk <= i + 2 and blk <= niter + 1
                        assert 0 <= 4 * q and 4 * q + 11 < UWW
                        assert pwoff + 4 * q + 3 < pww
                        assert 4 * q + 3 < SW  # stress ring write
                        x = x0 - 4 + 4 * q
                        if 0 <= j < nz and z0 <= j < z1 and 1 <= q <= 30 and x < nx:
                            o = origin + j * pitch + x
                            assert 0 <= o and o + 3 < elems
                            assert ((XPAD + x) * es) % min(16, 4 * es) == 0
                        # velocity phase
                        a = z0 - 8 + 4 * i + g
                        if a >= z0 and a < nz and 1 <= q <= 30 and x < nx:
                            assert i >= 2
                            blk = (a - (z0 - 8)) // 4
                            assert blk == i
                            for r in (a - 4, a + 4):
                                ii = (r - (z0 - 4)) // 4
                                assert i - 2 <= ii <= i  # held by the stress ring
                            assert 0 <= 4 * q - 4 and 4 * q + 7 < SW
                            o = origin + a * pitch + x
                            assert 0 <= o and o + 3 < elems


SIZES = [(96, 96), (96, 64), (250, 130), (257, 131), (500, 300), (1000, 1000), (1024, 1024),
         (2048, 1024), (4000, 2000), (800, 400), (16000, 8000), (1000, 500), (3999, 1999)]


@pytest.mark.parametrize("nx,nz", SIZES)
@pytest.mark.parametrize("es,wave", [(4, "psv"), (8, "psv"), (2, "psv"), (4, "sh"), (2, "sh")])
def test_fused_addresses_in_bounds(nx, nz, es, wave):
    per_sm = 1 if es == 8 else 3
    audit(nx, nz, es, wave, per_sm=per_sm)
    audit(nx, nz, es, wave, per_sm=per_sm, oversub=3.0)


def test_batch_plan_in_bounds():
    """The 64-shot batch of the benchmark under every autotuner candidate:
    every CTA serves one shot, and every shot's items pass the audit."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    F = pytest.importorskip("fd23_gb300")
    try:
        F.lib()
    except ImportError as e:
        pytest.skip(str(e))
    grids = [(d["nx"], d["nz"], 40, 0) for d in bench.batch_shots()]
    for wx, wz in ((1.0, 1.0), (2.5, 1.5), (4.0, 3.0), (6.0, 4.0), (4.0, 2.0), (3.0, 3.0)):
        for ov in (1.0, 2.0, 3.0):
            ctas = F.work_plan(grids, wx=wx, wz=wz, oversub=ov)
            assert len(ctas) % 456 == 0
            per_shot = {}
            for cta in ctas:
                shots = {it[0] for it in cta}
                assert len(shots) == 1
                per_shot.setdefault(cta[0][0], []).append([it[1:] for it in cta])
            assert sorted(per_shot) == list(range(len(grids)))
            if (wx, wz, ov) == (4.0, 3.0, 1.0):
                for k, c in per_shot.items():
                    audit(grids[k][0], grids[k][1], 4, "psv", ctas=c)
