"""CPU audit of every address the fused sweep forms (fd23_gb300/csrc/fd23_fused.cuh).

Takes the work plans from the library (fd23_work_plan: the planner the
solver and the batch use), restates the padded layout (make_layout) and the
index arithmetic of the kernel, then checks, for the grid sizes the tests and
the benchmarks use (and the 64-shot batch), that

  * every tensor copy (a box [fields][4 rows][width] of a 3-D view
    [field][row][column] of a padded block) lies inside the tensor's
    extents, starts at an x coordinate whose byte offset is a multiple of 16,
    moves rows of a multiple of 16 bytes, and lands on a 128-byte aligned
    shared-memory address;
  * every shared-memory read and write stays inside its ring;
  * every HBM store lands on a cell of the grid;
  * no CTA holds more work items than its item table;
  * the uniform fast iterations of the 16-bit sweep take only warps whose
    lanes are all interior, on z-interior rows of their item.

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


def worklist(nx, nz, npml, oversub=1.0, per_sm=3, bands=0):
    F = pytest.importorskip("fd23_gb300")
    try:
        F.lib()
    except ImportError as e:
        pytest.skip(str(e))
    return [[it[1:] for it in cta]
            for cta in F.work_plan([(nx, nz, npml, 0)], per_sm=per_sm, oversub=oversub, bands=bands)]


def al128(b):
    return (b + 127) // 128 * 128


def smem_layout(es, wave):
    """Byte offsets of the ring slots / stage groups (Cfg in fd23_fused.cuh)."""
    nv, nt = (2, 3) if wave == "psv" else (1, 2)
    nms, nmv = (3, 2) if wave == "psv" else (2, 1)
    pwoff = 4 if es == 2 else 0
    pww = SW + 2 * pwoff
    uw_slot = al128(nv * 4 * UWW * es)
    pg_ms = al128(nt * 4 * pww * es)
    pg_mv = pg_ms + al128(nms * 4 * pww * es)
    stage = pg_mv + al128(nmv * 4 * pww * es)
    return dict(nv=nv, nt=nt, nms=nms, nmv=nmv, pwoff=pwoff, pww=pww, uw_slot=uw_slot, pg_ms=pg_ms,
                pg_mv=pg_mv, stage=stage, pw_base=NUW * uw_slot)


def box_ok(x, y, z, w, nf, pitch, rows, nfields, es):
    # a copy may start left of the array (strips whose origin lies left of
    # column 0) or end past its last column: those elements read as zero,
    # as the padding columns hold; it must overlap the array
    assert x + w > 0 and x < pitch, (x, w, pitch)
    assert y >= 0 and y + 4 <= rows, (y, rows)
    assert z >= 0 and z + nf <= nfields
    assert (x * es) % 16 == 0 and (w * es) % 16 == 0
    assert w <= 256 and nf <= 256


def audit(nx, nz, es, wave, per_sm=3, oversub=1.0, ctas=None, narrowed=False, bands=0):
    pitch, rows, origin = layout(nx, nz)
    npml = min(40, nx // 2, nz // 2)
    elems = pitch * rows
    lay = smem_layout(es, wave)
    nfld = 5 if wave == "psv" else 3
    for off in [k * lay["uw_slot"] for k in range(NUW)] + \
               [lay["pw_base"] + g * lay["stage"] + o for g in range(NPW) for o in (0, lay["pg_ms"], lay["pg_mv"])]:
        assert off % 128 == 0
    nv = 2 if wave == "psv" else 1
    nt = 3 if wave == "psv" else 2
    npf = 8 if wave == "psv" else 5
    pwoff = 4 if es == 2 else 0
    pww = SW + 2 * pwoff
    assert (pitch * es) % 16 == 0
    if ctas is None:
        ctas = worklist(nx, nz, npml, oversub, per_sm, bands)
    covered = set()
    # strip origin: a multiple of 8 in (-TX, 0], congruent to every x0 mod TX
    r = min(x0 for items in ctas for (x0, _, _) in items) % TX if any(ctas) else 0
    xoff = r - TX if r else 0
    assert -TX < xoff <= 0 and xoff % 8 == 0
    for items in ctas:
        assert (0 if narrowed else 1) <= len(items) <= MAX_ITEMS
        for (x0, z0, z1) in items:
            for zb in range(z0 // 4, z1 // 4):
                key = (x0, zb)
                assert key not in covered  # every block exactly once
                covered.add(key)
        for (x0, z0, z1) in items:
            assert (x0 - xoff) % TX == 0 and z0 % 4 == 0 and z1 % 4 == 0 and z1 > z0
            niter = (z1 - z0) // 4 + 2
            # stencil-input copies: blocks 0 .. niter+1, rows z0-8+4b .. +3
            for b in (0, niter + 1):
                box_ok(XPAD + x0 - 8, ZPAD + z0 - 8 + 4 * b, 0, UWW, lay["nv"], pitch, rows, nfld, es)
            # point-wise copies of iterations 0 .. niter-1: old stresses and
            # stress-update material on stress rows, velocity-update material
            # on velocity rows
            for i in (0, niter - 1):
                xs = XPAD + x0 - 4 - lay["pwoff"]
                box_ok(xs, ZPAD + z0 - 4 + 4 * i, lay["nv"], lay["pww"], lay["nt"], pitch, rows, nfld, es)
                box_ok(xs, ZPAD + z0 - 4 + 4 * i, 0, lay["pww"], lay["nms"], pitch, rows, nfld, es)
                box_ok(xs, ZPAD + z0 - 8 + 4 * i, lay["nms"], lay["pww"], lay["nmv"], pitch, rows, nfld, es)
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
                        if 0 <= j < nz and z0 <= j < z1 and 1 <= q <= 30 and 0 <= x < nx:
                            o = origin + j * pitch + x
                            assert 0 <= o and o + 3 < elems
                            assert ((XPAD + x) * es) % min(16, 4 * es) == 0
                        # velocity phase
                        a = z0 - 8 + 4 * i + g
                        if a >= z0 and a < nz and 1 <= q <= 30 and 0 <= x < nx:
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
    per_sm = {8: 1, 4: 3, 2: 2}[es]  # the register budget each storage width is built for
    for bands in (0, 1):  # strip-major and banded plans
        audit(nx, nz, es, wave, per_sm=per_sm, bands=bands)
        if es == 2:  # and three, should the runtime report three resident CTAs
            audit(nx, nz, es, wave, per_sm=3, bands=bands)
        audit(nx, nz, es, wave, per_sm=per_sm, oversub=3.0, bands=bands)


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
            ctas = F.work_plan(grids, wx=wx, wz=wz, oversub=ov, bands=0)
            assert len(ctas) % 456 == 0
            # banded: shots with fewer CTAs than strips keep the strip-major cut
            assert len(F.work_plan(grids, wx=wx, wz=wz, oversub=ov, bands=1)) <= len(ctas)
            per_shot = {}
            for cta in ctas:
                shots = {it[0] for it in cta}
                assert len(shots) == 1
                per_shot.setdefault(cta[0][0], []).append([it[1:] for it in cta])
            assert sorted(per_shot) == list(range(len(grids)))
            if (wx, wz, ov) == (4.0, 3.0, 1.0):
                for k, c in per_shot.items():
                    audit(grids[k][0], grids[k][1], 4, "psv", ctas=c)


def narrow(nx, nz, items, first, last, it, terms=()):
    """The item narrowing of the sweep with tile step windows (the PUNCH
    prologue of fused_step), restated: keep the rows from the first to the
    last tile row with a tile that is not steady at step it (or holds a
    source term, while it <= the source length), drop empty items."""
    nbx = (nx + 31) // 32

    def steady(t):
        f, l = int(first[t]), int(last[t])
        return not (f < it <= l and l - f >= 2)

    out = []
    for (x0, z0, z1) in items:
        rows = [tz for tz in range(z0 // 16, (min(z1, nz) - 1) // 16 + 1)
                if any(not steady(tz * nbx + tx) for tx in range(max(x0, 0) // 32, (min(x0 + TX, nx) - 1) // 32 + 1))]
        rows += [tz // 16 for (tx, tz) in terms if x0 <= tx < x0 + TX and z0 <= tz < z1]
        if not rows:
            continue
        a, b = max(z0, min(rows) * 16), min(z1, (max(rows) + 1) * 16)
        assert z0 <= a < b <= z1 and a % 4 == 0 and b % 4 == 0
        out.append((x0, a, b))
    return out


@pytest.mark.parametrize("nx,nz", [(230, 150), (256, 160), (700, 380), (2000, 1000), (4000, 2000)])
@pytest.mark.parametrize("es,wave", [(4, "psv"), (8, "psv"), (2, "sh")])
def test_narrowed_items_in_bounds(nx, nz, es, wave):
    """Items narrowed by random tile step windows keep every address of the
    audit in bounds (they are sub-ranges of plan items on 4-row blocks)."""
    import numpy as np
    rng = np.random.default_rng(nx + nz + es)
    nb = ((nx + 31) // 32) * ((nz + 15) // 16)
    first = rng.integers(-3, 60, size=nb)
    last = first + rng.integers(-2, 80, size=nb)
    npml = min(40, nx // 2, nz // 2)
    per_sm = {8: 1, 4: 3, 2: 2}[es]
    for ov in (1.0, 3.0):
        ctas = worklist(nx, nz, npml, ov, per_sm)
        for it in (0, 7, 31, 90):
            nar = [narrow(nx, nz, items, first, last, it, terms=[(nx // 2, nz // 3)]) for items in ctas]
            audit(nx, nz, es, wave, per_sm=per_sm, ctas=nar, narrowed=True)


@pytest.mark.parametrize("nx,nz", SIZES)
@pytest.mark.parametrize("es,wave", [(4, "psv"), (8, "psv"), (2, "psv"), (4, "sh"), (2, "sh")])
def test_table_index_box_in_bounds(nx, nz, es, wave):
    """The material-table form copies, per iteration, 8 index rows (bytes)
    of kIdxBoxW = 160 from the 16-byte boundary at or before the point-wise
    copy's start: x is a multiple of 16 bytes, the rows lie inside the
    padded index array, every thread's 4 index bytes lie inside the box and
    are 4-byte aligned, and the stage layout stays 128-byte aligned.  Index
    bytes of columns left of the array (strips whose origin lies left of
    column 0) read as index 0: those cells are outside the grid, their
    results are never stored."""
    IW = 160
    pitch, rows, origin = layout(nx, nz)
    lay = smem_layout(es, wave)
    npml = min(40, nx // 2, nz // 2)
    pg_ms = lay["pg_ms"]
    stage = pg_ms + al128(8 * IW)
    assert pg_ms % 128 == 0 and stage % 128 == 0
    for items in worklist(nx, nz, npml, 1.0, {8: 1, 4: 3, 2: 2}[es]):
        for (x0, z0, z1) in items:
            niter = (z1 - z0) // 4 + 2
            xs = XPAD + x0 - 4 - lay["pwoff"]
            xa = xs & ~15
            # left of the array (a strip origin left of column 0) the copy reads zeros
            assert xa + IW > 0 and xa % 16 == 0 and xa <= xs
            for i in (0, niter - 1):
                yv = ZPAD + z0 - 8 + 4 * i
                assert yv >= 0 and yv + 8 <= rows
            for q in (0, 31):
                ixo = (xs & 15) + lay["pwoff"] + 4 * q
                assert ixo % 4 == 0 and ixo + 3 < IW
                # the byte is the cell the point-wise row holds at this lane
                assert xa + ixo == XPAD + x0 - 4 + 4 * q


@pytest.mark.parametrize("nx,nz", [(230, 150), (1000, 500), (4000, 2000), (257, 131)])
@pytest.mark.parametrize("density", [0.0, 0.05, 0.3, 1.0])
def test_live_mask_plans(nx, nz, density):
    """Plans over live blocks (the phase plans of the windowed sweep): every
    live 4-row block is planned exactly once and nothing else, items stay in
    one strip on whole blocks, no CTA has more than 4 items, the addresses
    pass the audit, and an all-live mask gives the ordinary plan."""
    import numpy as np
    F = pytest.importorskip("fd23_gb300")
    try:
        F.lib()
    except ImportError as e:
        pytest.skip(str(e))
    ntx, nzb = (nx + TX - 1) // TX, (nz + 3) // 4
    rng = np.random.default_rng(nx + int(100 * density))
    # live regions shaped like a growing wavefront, plus scattered blocks
    zz, xx = np.mgrid[0:nzb, 0:ntx]
    live = (np.hypot((xx - ntx / 2) * 30, zz * 4) < density * 2 * max(nx, nz)) | (rng.random((nzb, ntx)) < density / 10)
    mask = live.T.ravel()  # strip-major
    npml = min(40, nx // 2, nz // 2)
    for ov in (1.0, 3.0):
        ctas = F.work_plan([(nx, nz, npml, 0)], wx=5.0, wz=4.0, oversub=ov, live=[mask])
        seen = np.zeros(ntx * nzb, int)
        for cta in ctas:
            assert len(cta) <= MAX_ITEMS
            for (_, x0, z0, z1) in cta:
                assert x0 % TX == 0 and z0 % 4 == 0 and z1 % 4 == 0 and z1 > z0
                for zb in range(z0 // 4, z1 // 4):
                    seen[(x0 // TX) * nzb + zb] += 1
        np.testing.assert_array_equal(seen, mask.astype(int))
        if mask.any():
            audit(nx, nz, 4, "psv", ctas=[[it[1:] for it in c] for c in ctas], narrowed=True)
    full = F.work_plan([(nx, nz, npml, 0)], wx=5.0, wz=4.0, live=[np.ones(ntx * nzb, bool)])
    plain = F.work_plan([(nx, nz, npml, 0)], wx=5.0, wz=4.0, bands=0)
    # masks are laid out over strips from column 0; the ordinary plan may move
    # its origin left (then only the block coverage is the same)
    if min(it[1] for cta in plain for it in cta) == 0:
        assert full == plain
    else:
        assert all(it[1] % TX == 0 for cta in full for it in cta)


@pytest.mark.parametrize("nx,nz,npml", [(4000, 2000, 40), (16000, 8000, 40), (800, 400, 20), (1000, 1000, 20),
                                        (257, 131, 12)])
@pytest.mark.parametrize("ov", [1.0, 3.0])
def test_banded_plan_covers_grid_with_shared_row_cuts(nx, nz, npml, ov):
    """Banded plans (fd23_tune_entry.bands = 1): one item per CTA, every
    4-row block of the grid exactly once, no more CTAs than the strip-major
    plan, and every interior strip cut at the same rows (the x-CPML strips
    have their own cut); their copies pass the audit."""
    F = pytest.importorskip("fd23_gb300")
    try:
        F.lib()
    except ImportError as e:
        pytest.skip(str(e))
    ref = F.work_plan([(nx, nz, npml, 0)], wx=5.0, wz=2.5, oversub=ov, bands=0)
    ctas = F.work_plan([(nx, nz, npml, 0)], wx=5.0, wz=2.5, oversub=ov, bands=1)
    if len(ref) < len({it[1] for cta in ref for it in cta}):  # fewer CTAs than strips: strip-major
        assert ctas == ref
        return
    assert len(ctas) <= len(ref)
    cuts = {}
    for cta in ctas:
        assert len(cta) == 1
        (_, x0, z0, z1), = cta
        cuts.setdefault(x0, []).append((z0, z1))
    xoff = min(cuts)
    assert -TX < xoff <= 0 and xoff % 8 == 0
    ntx = (nx - xoff + TX - 1) // TX
    assert sorted(cuts) == [xoff + TX * s for s in range(ntx)]
    nzb = (nz + 3) // 4
    for x0, c in cuts.items():
        c.sort()
        assert c[0][0] == 0 and c[-1][1] == 4 * nzb
        assert all(a[1] == b[0] for a, b in zip(c, c[1:]))
    interior = [x0 for x0 in cuts if x0 - 4 >= max(npml, 4) and x0 + TX + 4 <= min(nx - npml, nx - 4)]
    assert len({tuple(cuts[x0]) for x0 in interior}) <= 1
    audit(nx, nz, 4, "psv", ctas=[[it[1:] for it in cta] for cta in ctas])


def _xp_strips(nx, npml, x0s):
    """strips whose 128 stress columns reach the x-CPML or the reduced-order
    edge columns (the planner's x-CPML strips)"""
    return [x0 for x0 in x0s if x0 - 4 < max(npml, 4) or x0 + TX + 4 > min(nx - npml, nx - 4)]


@pytest.mark.parametrize("nx,nz,npml,want_xp", [(4000, 2000, 40, 2), (16000, 8000, 40, 2), (2000, 1000, 40, 2),
                                                 (800, 400, 20, 2)])
def test_strip_origin_puts_the_cpml_into_fewest_strips(nx, nz, npml, want_xp):
    """The planner moves the strips' origin left of column 0 (a multiple of
    8 above -120) when that puts the x-CPML zones and their halos into fewer
    strips: on the 4000-column grid with a 40-cell CPML, two CPML strips
    (origin 0 gives three: 0, 32 and 33)."""
    F = pytest.importorskip("fd23_gb300")
    try:
        F.lib()
    except ImportError as e:
        pytest.skip(str(e))
    for bands in (0, 1):
        ctas = F.work_plan([(nx, nz, npml, 0)], wx=5.0, wz=2.5, bands=bands)
        x0s = sorted({it[1] for cta in ctas for it in cta})
        xoff = x0s[0]
        assert -TX < xoff <= 0 and xoff % 8 == 0
        assert x0s == [xoff + TX * s for s in range(len(x0s))] and x0s[-1] + TX >= nx
        assert len(_xp_strips(nx, npml, x0s)) == want_xp
        # no origin puts the CPML into fewer strips
        for xo in range(0, -TX, -8):
            cand = [xo + TX * s for s in range((nx - xo + TX - 1) // TX)]
            assert len(_xp_strips(nx, npml, cand)) >= want_xp
    if (nx, npml) == (4000, 40):
        import numpy as np
        ref = F.work_plan([(nx, nz, npml, 0)], wx=5.0, wz=2.5, bands=0, live=[np.ones(34 * ((nz + 3) // 4), bool)])
        assert len(_xp_strips(nx, npml, sorted({it[1] for cta in ref for it in cta}))) == 3


@pytest.mark.parametrize("es,wave", [(4, "psv"), (2, "psv"), (4, "sh"), (2, "sh")])
@pytest.mark.parametrize("batch", [False, True])
def test_three_ctas_fit_per_sm(es, wave, batch):
    """Dynamic shared memory of the sweep (Cfg::SMEM in fd23_fused.cuh: the
    two rings and the point-wise stages in the storage type, the stress ring
    in the arithmetic type (4-byte floats for every form but FP64), with
    16-bit storage the strip's x-CPML coefficient table, barriers,
    item and source-term tables), its static shared memory (the batched
    sweep's copy of the descriptor head) and the 1 KB the runtime reserves
    per CTA: three CTAs fit the 228 KB of one SM."""
    lay = smem_layout(es, wave)
    nt = lay["nt"]
    ring = NUW * lay["uw_slot"] + NPW * lay["stage"] + NTR * 4 * nt * SW * 4
    if es == 2:
        ring += 12 * SW * 4  # the strip's x-CPML coefficients (b, c, k at 4 positions)
    smem = (ring + 15) // 16 * 16 + 256 + MAX_ITEMS * 16 + MAX_ITEMS * 16 * 16
    static = 512 if batch else 128
    assert 3 * (smem + static + 1024) <= 228 * 1024, (smem, static)


@pytest.mark.parametrize("nx,nz,npml", [(60, 40, 0), (100, 64, 0), (130, 97, 10), (121, 33, 4), (500, 300, 0),
                                        (4000, 2000, 0)])
@pytest.mark.parametrize("bands", [0, 1])
@pytest.mark.parametrize("ov", [1.0, 2.0])
def test_plans_without_cpml_and_narrow_grids(nx, nz, npml, bands, ov):
    """Grids without a CPML (only the reduced-order edge columns cost more),
    grids narrower than one strip, and a strip boundary at the grid's edge:
    every 4-row block planned once, copies and stores in bounds."""
    F = pytest.importorskip("fd23_gb300")
    try:
        F.lib()
    except ImportError as e:
        pytest.skip(str(e))
    ctas = F.work_plan([(nx, nz, npml, 0)], wx=5.0, wz=2.5, oversub=ov, bands=bands)
    items = [it[1:] for cta in ctas for it in cta]
    x0s = sorted({x0 for x0, _, _ in items})
    xoff = x0s[0]
    assert -TX < xoff <= 0 and xoff % 8 == 0
    assert x0s == [xoff + TX * s for s in range(len(x0s))] and x0s[-1] + TX >= nx
    nzb = (nz + 3) // 4
    seen = {}
    for x0, z0, z1 in items:
        for zb in range(z0 // 4, z1 // 4):
            seen[(x0, zb)] = seen.get((x0, zb), 0) + 1
    assert len(seen) == len(x0s) * nzb and set(seen.values()) == {1}
    audit(nx, nz, 4, "psv", ctas=[[it[1:] for it in cta] for cta in ctas])


@pytest.mark.parametrize("nx,nz,npml,top", [(4000, 2000, 40, 0), (1000, 500, 20, 1), (500, 260, 0, 0),
                                            (140, 200, 8, 0), (16000, 8000, 40, 0)])
@pytest.mark.parametrize("bands", [0, 1])
def test_fast_iterations_are_interior(nx, nz, npml, top, bands):
    """The fast-iteration test of the single-shot 16-bit sweep (fd23_fused.cuh:
    item_fast, fjlo, fjhi) restated.  On every warp-iteration it accepts, every
    lane of the warp is x-interior and the stress row and the velocity row are
    z-interior, so the per-lane path would take its interior branches for all
    of them, and the velocity row belongs to the item (the fast stores check
    only j < z1 and the owned lanes).  A source term in an item only removes
    fast iterations.  On the benchmark grids most warp-iterations are fast."""
    ctas = worklist(nx, nz, npml, 1.0, 3, bands)

    def xfast(x):
        return x >= max(4, npml) and x + 3 <= min(nx - 5, nx - npml - 1)

    def zfast(j):
        return 4 <= j <= nz - 5 and j < nz - npml and not (top and j < npml)

    fast = total = 0
    for items in ctas:
        for (x0, z0, z1) in items:
            niter = (z1 - z0) // 4 + 2
            lanes_x = [x0 - 4 + 4 * q for q in range(32)]
            item_fast = all(xfast(x) for x in lanes_x)
            fjlo = max(z0, max(4, npml if top else 0)) + 4 if item_fast else 2 ** 31 - 1
            fjhi = min(nz - 5, nz - npml - 1)
            for i in range(niter):
                for g in range(4):
                    total += 1
                    j = z0 - 4 + 4 * i + g
                    if not fjlo <= j <= fjhi:
                        continue
                    fast += 1
                    a = j - 4
                    assert zfast(j) and zfast(a) and z0 <= a < nz and j >= z0
                    assert all(xfast(x) and 0 <= x and x + 3 < nx for x in lanes_x)
    if nx >= 4000:
        assert fast > 0.75 * total, (fast, total)
