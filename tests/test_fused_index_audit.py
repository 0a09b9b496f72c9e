"""CPU audit of every address the fused sweep forms (fd23_gb300/csrc/fd23_fused.cu).

Restates the work-list construction (fd23_api.cpp: build_worklist,
make_layout) and the index arithmetic of the kernel, then checks, for the
grid sizes the tests and the benchmark use, that

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


def worklist(nx, nz, sms=152, per_sm=2, npml=40, wx=4.0, wz=3.0, top=False):
    """Cost-weighted contiguous partition of the 4-row blocks (build_worklist)."""
    import bisect
    ntx = (nx + TX - 1) // TX
    nzb = (nz + 3) // 4
    total = ntx * nzb
    nb = min(sms * per_sm, total)
    nb = max(nb, (ntx + 1) // 2)
    cum = [0.0]
    for b in range(total):
        strip, zb = divmod(b, nzb)
        x0 = strip * TX
        xp = (x0 - 4 < max(npml, 4)) or (x0 + TX + 4 > min(nx - npml, nx - 4))
        r0, r1 = 4 * zb, 4 * zb + 3
        zp = (r1 >= min(nz - npml, nz - 4)) or r0 < 4 or (top and r0 < npml)
        cum.append(cum[-1] + (wx if xp else (wz if zp else 1.0)))
    ctas = []
    b0 = 0
    for c in range(nb):
        if c == nb - 1:
            b1 = total
        else:
            target = cum[total] * (c + 1) / nb
            b1 = bisect.bisect_left(cum, target, b0 + 1)
            b1 = max(b1, b0 + 1)
            b1 = min(b1, total - (nb - 1 - c))
        items = []
        while b0 < b1:
            strip = b0 // nzb
            e = min(b1, (strip + 1) * nzb)
            items.append((strip * TX, (b0 - strip * nzb) * 4, (e - strip * nzb) * 4))
            b0 = e
        ctas.append(items)
    assert b0 == total
    return ctas


def audit(nx, nz, es, wave, sms=152, per_sm=2):
    pitch, rows, origin = layout(nx, nz)
    npml = min(40, nx // 2, nz // 2)
    elems = pitch * rows
    nv = 2 if wave == "psv" else 1
    nt = 3 if wave == "psv" else 2
    npf = 8 if wave == "psv" else 5
    pwoff = 4 if es == 2 else 0
    pww = SW + 2 * pwoff
    assert (pitch * es) % 16 == 0
    for items in worklist(nx, nz, sms, per_sm, npml=npml):
        assert 1 <= len(items) <= MAX_ITEMS
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
