"""CPU audit of every address the two-step sweep forms (fd23_gb300/csrc/fd23_fused2.cu).

Restates the padded layout (make_layout), the strip geometry (232 output
columns per strip, rows [z0, z1) in 4-row blocks, phases reaching 16 rows
above and below) and the kernel's index arithmetic, and checks, for the grid
sizes the tests and the benchmarks use, that

  * every tensor copy starts on a 16-byte boundary of its x dimension (the
    264-column input rows through a 4-D view whose copies start on an
    8-column group), has box dimensions of at most 256 elements, and lands on
    a 128-byte aligned shared-memory offset; rows outside the array are the
    copy's zero fill;
  * every read of the second step's material through the read-only path and
    every HBM store of the step-(it+2) wavefields lies inside the padded
    array and is aligned for its vector width;
  * every memory-variable index of a CPML cell lies inside its array;
  * every shared-memory read and write of the rings and stages stays inside
    its region, and the regions fit the 227 KB a CTA may hold.

Index expressions are affine in the column group t (0..63) and the row, so
the extreme values bound every thread.
"""
import pytest

XPAD = ZPAD = 8
TX1 = 120                  # one-step strips (they size the layout)
WIDTHS = (256, 128)        # two-step sweep: ring row width W1; output columns W1 - 24
NUW, NPW, NR = 4, 2, 3

GRIDS = [(96, 64, 12), (250, 130, 12), (257, 131, 16), (300, 200, 12), (130, 97, 12), (700, 90, 12),
         (1000, 1000, 20), (200, 120, 12), (180, 140, 12), (600, 300, 20), (2000, 1000, 40),
         (4000, 2000, 40), (16000, 8000, 40)]


def layout(nx, nz):
    ntx = (nx + TX1 - 1) // TX1
    cover_x, cover_z = ntx * TX1, (nz + 3) // 4 * 4
    pitch = (XPAD + max(cover_x, nx) + 8 + 31) // 32 * 32
    rows = ZPAD + max(cover_z, nz) + 8
    return pitch, rows, ZPAD * pitch + XPAD


def al128(b):
    return (b + 127) // 128 * 128


def smem(es_mat, W1):
    uww = W1 + 8
    moff = 4 if es_mat == 2 else 0
    mww = W1 + 2 * moff
    uw_slot = 4 * uww * 4          # 4 rows of one field: U and W rings of NUW slots each
    told = 3 * 4 * W1 * 4
    ms_b, mv_b = al128(3 * 4 * mww * es_mat), al128(2 * 4 * mww * es_mat)
    stage = told + ms_b + mv_b
    off_pw = 2 * NUW * uw_slot
    off_tr = off_pw + NPW * stage
    off_vr = off_tr + NR * 4 * 3 * W1 * 4
    off_t2 = off_vr + NR * 4 * 2 * W1 * 4
    off_bar = off_t2 + NR * 4 * 3 * W1 * 4
    total = off_bar + 128 + 4 * 16 + 4 * 16 * 16
    return dict(moff=moff, mww=mww, uw_slot=uw_slot, told=told, ms_b=ms_b, mv_b=mv_b, stage=stage,
                off_pw=off_pw, off_tr=off_tr, off_vr=off_vr, off_t2=off_t2, total=total)


@pytest.mark.parametrize("W1", WIDTHS)
@pytest.mark.parametrize("es_mat", [4, 2])
def test_shared_memory_regions(es_mat, W1):
    m = smem(es_mat, W1)
    UWW = W1 + 8
    per_sm = 256 // W1
    # the CTAs per SM the launch bounds promise fit in 228 KB (1 KB reserved per CTA)
    assert per_sm * (m["total"] + 1024) <= 228 * 1024
    for k in ("off_pw", "off_tr", "off_vr", "off_t2", "stage", "uw_slot"):
        assert m[k] % 128 == 0, k
    assert (m["told"] + m["ms_b"]) % 128 == 0
    # box dimensions: input {8, UWW/8, 4, 1}; stresses {W1, 4, 3}; material {mww, 4, 3|2}
    assert UWW % 8 == 0 and UWW // 8 <= 256
    assert W1 <= 256
    if es_mat == 4:
        assert m["mww"] <= 256
    # bytes a stage's copies deliver equal the stage's expect_tx
    assert m["told"] + 5 * 4 * m["mww"] * es_mat <= m["stage"]
    # ring reads: ld12 reads p-4 .. p+7 of a row, p = 4t (rings) or 4 + 4t (input rows)
    ntr = W1 // 4
    for lo, hi in ((1, ntr - 2), (2, ntr - 3), (3, ntr - 4)):  # V1, S2, V2 read rings
        assert 4 * lo - 4 >= 0 and 4 * hi + 7 < W1
    assert 4 * (ntr - 1) + 4 + 7 < UWW and 0 + 4 - 4 >= 0  # S1 reads input rows
    # writes: S1 all groups, V1 / S2 their ranges, all inside a ring row
    assert 4 * (ntr - 1) + 3 < W1
    # material rows in a stage: offset moff + 4t
    assert m["moff"] + 4 * (ntr - 1) + 3 < m["mww"]
    # 12-row ring rows: rb + d with rb < 12, d <= 8 wraps at most once
    assert all((rb + d if rb + d < 12 else rb + d - 12) < 12 for rb in range(12) for d in range(9))


@pytest.mark.parametrize("W1", WIDTHS)
@pytest.mark.parametrize("nx,nz,npml", GRIDS)
def test_global_addresses(nx, nz, npml, W1):
    pitch, rows, origin = layout(nx, nz)
    elems = pitch * rows
    assert pitch % 32 == 0 and pitch % 8 == 0
    assert elems < 2 ** 31  # 32-bit element offsets
    TX = W1 - 24
    ntr = W1 // 4
    nstrip = (nx + TX - 1) // TX
    for s in range(nstrip):
        x0 = s * TX
        # input copy: 8-column group coordinate, whole groups
        xs = XPAD + x0 - 16
        assert xs % 8 == 0
        # stress / material copies: 16-byte x starts for FP32, 8-column starts for FP16
        assert ((XPAD + x0 - 12) * 4) % 16 == 0
        assert (XPAD + x0 - 12 - 4) % 8 == 0
        for t_lo, t_hi in ((2, ntr - 3), (3, ntr - 4)):
            for t in (t_lo, t_hi):
                x = x0 - 12 + 4 * t
                if not (x + 3 >= 0 and x < nx):
                    continue
                for j in (0, nz - 1):
                    a = origin + j * pitch + x
                    assert a % 4 == 0 and a >= 0 and a + 3 < elems
        # owned HBM stores: x in [x0, x0 + TX) and < nx, rows [0, nz)
        xl, xh = x0, min(x0 + TX, nx) - 1
        for x in (xl, xh):
            for j in (0, nz - 1):
                a = origin + j * pitch + x
                assert 0 <= a < elems
    # the zero rows above and below the grid that the sweep reads as values:
    # rows -8 .. -1 and nz .. nz+7 are padding (zero); beyond, the copy's fill
    assert rows >= ZPAD + nz + 8


@pytest.mark.parametrize("nx,nz,npml", GRIDS)
def test_memory_variable_indices(nx, nz, npml):
    nxp, nzp = 2 * npml * nz, 2 * npml * nx  # x- and z-CPML arrays
    for top in (0, 1):
        for ix in (0, npml - 1, nx - npml, nx - 1):
            for j in (0, nz - 1):
                if ix < npml or ix >= nx - npml:
                    px = ix + j * 2 * npml if ix < npml else npml + nx - 1 - ix + j * 2 * npml
                    assert 0 <= px < nxp
        for j in (0, npml - 1, nz - npml, nz - 1):
            for ix in (0, nx - 1):
                is_top = j < npml and top
                if is_top or j >= nz - npml:
                    pz = j * nx + ix if is_top else (npml + nz - 1 - j) * nx + ix
                    assert 0 <= pz < nzp
    # the z-CPML interior branch reads 4 consecutive cells from x >= max(4, npml)
    # up to x + 3 <= min(nx - 5, nx - npml - 1)
    xh = min(nx - 5, nx - npml - 1) - 3
    for j, is_top in ((npml - 1, True), (nz - npml, False), (nz - 5, False)):
        pz0 = j * nx + xh if is_top else (npml + nz - 1 - j) * nx + xh
        assert 0 <= pz0 and pz0 + 3 < nzp
