"""Hybrid box, CPU side: ring geometry and the FP64 host builders against the
oracle, and the oracle's box run against its own plain run (a box driven by
the ring field of a recorded run must reproduce that run outside the box)."""
import numpy as np
import pytest

from oracle import fd23_oracle as O
from tests.fd23_cases import Case

F = pytest.importorskip("fd23_gb300")


def _lib_or_skip():
    try:
        F.lib()
    except ImportError as e:  # library not built
        pytest.skip(str(e))


def reference_square_rings(bw, xs, zs, nx):
    """The ring loops of PD/box/box.cpp:26-95 for a bw x bw box around
    (xs, zs), written out independently of the oracle."""
    idxend = (bw + 1) // 2
    idxstart = idxend + 1 - bw
    s0 = idxstart
    s1, s2, s3 = s0 + 3, s0 + 4, s0 + 7
    s7 = idxend
    s6, s5, s4 = s7 - 3, s7 - 4, s7 - 7
    xs_b = zs_b = -idxstart
    sub_r, sub_a, add_r, add_a = [], [], [], []
    for j in range(s0, s7 + 1):
        for i in range(s0, s7 + 1):
            if not (s1 < i < s6 and s1 < j < s6):
                sub_r.append((j + zs_b) * bw + i + xs_b)
                sub_a.append((j + zs) * nx + i + xs)
    for j in range(s2, s5 + 1):
        for i in range(s2, s5 + 1):
            if not (s3 < i < s4 and s3 < j < s4):
                add_r.append((j + zs_b) * bw + i + xs_b)
                add_a.append((j + zs) * nx + i + xs)
    return (np.array(sub_r + add_r), np.array(sub_a + add_a), len(sub_r), xs + idxstart,
            zs + idxstart)


@pytest.mark.parametrize("bw", [16, 21, 22, 31, 32])
def test_oracle_rings_match_reference_loops(bw):
    nx, xs, zs = 97, 48, 40
    rr, ra, nsub, x0, z0 = reference_square_rings(bw, xs, zs, nx)
    g, r, ns = O.box_rings(nx, x0, z0, bw, bw)
    assert ns == nsub
    np.testing.assert_array_equal(r, rr)
    np.testing.assert_array_equal(g, ra)


def test_ring_index_closed_form_matches_enumeration():
    _lib_or_skip()
    rng = np.random.default_rng(5)
    sizes = [(16, 16), (17, 16), (16, 40), (21, 21), (64, 33)]
    sizes += [tuple(int(v) for v in rng.integers(16, 90, size=2)) for _ in range(12)]
    for bx, bz in sizes:
        nx = bx + 7
        g, r, nsub = O.box_rings(nx, 3, 2, bx, bz)
        assert F.box_ring_size(bx, bz) == (nsub, len(g) - nsub)
        ix, iz = F.box_ring_cells(3, 2, bx, bz)
        np.testing.assert_array_equal(ix + iz * nx, g)
        pos = np.full(bx * bz, -1)
        pos[r] = np.arange(len(r))
        got = np.array([F.box_ring_index(bx, bz, i, j) for j in range(bz) for i in range(bx)])
        np.testing.assert_array_equal(got, pos)
    # the box of the hybrid-box workload: 2000 x 1000
    ns, na = F.box_ring_size(2000, 1000)
    assert (ns, na) == O.box_ring_count(2000, 1000)
    with pytest.raises(F.Fd23Error):
        F.box_ring_size(15, 40)


@pytest.mark.parametrize("bx,bz", [(21, 21), (24, 17)])
def test_incident_from_displacement_bit_exact(bx, bz):
    _lib_or_skip()
    rng = np.random.default_rng(bx * 100 + bz)
    planes = [rng.standard_normal((bz + 8, bx + 8)) * 1e-3 for _ in range(4)]
    bmat = rng.uniform(0.1, 1.0, size=(5, bz, bx))
    dt = 4e-4
    want = O.box_incident_from_displacement(bx, bz, dt, bmat, *planes)
    got = F.box_incident_from_displacement(bx, bz, dt, bmat, *planes)
    np.testing.assert_array_equal(got, want)
    # velocities are the plane difference over dt
    g, r, _ = O.box_rings(bx, 0, 0, bx, bz)
    bi, bj = r % bx, r // bx
    np.testing.assert_array_equal(got[0], (planes[2][bj + 4, bi + 4] - planes[0][bj + 4, bi + 4]) / dt)


def test_box_material_bit_exact():
    _lib_or_skip()
    c = Case("psv", 90, 70, npml=10, seed=4)
    x0, z0, bx, bz = 30, 20, 21, 21
    srcvp, srcvs, srcden = 5.0, 5.0 / 1.73, 0.31 * 5.0 ** 0.25 * 8.0
    m1, b1, n1 = O.box_material(c.mat, x0, z0, bx, bz, srcvp, srcvs, srcden, c.dt, c.h)
    m2, b2, n2 = F.box_material(c.mat, x0, z0, bx, bz, srcvp, srcvs, srcden, c.dt, c.h)
    assert n1 == n2 > 0
    np.testing.assert_array_equal(m1, m2)
    np.testing.assert_array_equal(b1, b2)
    # a second pass finds the box homogeneous already
    _, _, n3 = F.box_material(m2, x0, z0, bx, bz, srcvp, srcvs, srcden, c.dt, c.h)
    assert n3 == 0


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_oracle_box_reproduces_recorded_run(prec):
    """Self-consistency: record the ring field of a run with a source inside
    the box, drive a box run (no source) with it; everything outside the add
    ring's interior must match the recorded run bit for bit, and r stays 0."""
    nx, nz, nt = 120, 80, 70
    c = Case("psv", nx, nz, npml=10, nt=nt, xs=60, zs=30, seed=3)
    box = (30, 15, 60, 40)
    x0, z0, bx, bz = box
    inc, _ = O.psv_ring_history(prec, nx, nz, c.npml, 0, c.mat, c.bck, c.terms, nt, box)
    rmat = c.mat[:, z0:z0 + bz, x0:x0 + bx]
    rf = np.repeat(np.arange(5, dtype=np.int32), len(c.rec))
    ri = np.tile(c.rec, 5)
    none = (np.zeros(0, np.int32), np.zeros(0, np.int64), np.zeros((0, 1)))
    seis, st, rst = O.psv_box_run(prec, nx, nz, c.npml, 0, c.mat, c.bck, none, rf, ri, nt, box,
                                  rmat, inc)
    (su, sw), st_plain = c.oracle(prec)
    n = nx * nz
    keep = np.ones((nz, nx), bool)
    keep[z0 + 4:z0 + bz - 4, x0 + 4:x0 + bx - 4] = False
    for f in range(5):
        a = st[f * n:(f + 1) * n].reshape(nz, nx)
        b = st_plain[f * n:(f + 1) * n].reshape(nz, nx)
        np.testing.assert_array_equal(a[keep], b[keep])
    np.testing.assert_array_equal(st[5 * n:], st_plain[5 * n:])  # CPML memory variables
    assert not np.any(rst)
    out = keep[c.rz, c.rx]
    np.testing.assert_array_equal(seis[:, :len(c.rec)][:, out], su[:, out])
    np.testing.assert_array_equal(seis[:, len(c.rec):2 * len(c.rec)][:, out], sw[:, out])
