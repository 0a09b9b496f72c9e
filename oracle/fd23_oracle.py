"""Python front end of the fd23 CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It wraps ``libfd23_oracle.so`` (built from
``oracle/fd23_oracle.c`` by ``oracle/build.py``) with ctypes and adds the
small host-side pieces of the reference setup: the ``.mdl`` parser, the CPML
assignment table and the receiver pair duplication.

Reference citations are relative to the fd23 project root
(PD = PSV/psv_clean_double, PN = PSV/clean_nobox, SH = SH).
"""
import ctypes as C
import math
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        d, i, l, vp = C.c_double, C.c_int, C.c_long, C.c_void_p
        _lib.or_psv_material.argtypes = [i, i, d, d, vp, vp, vp, vp, vp]
        _lib.or_sh_material.argtypes = [i, i, d, d, vp, vp, vp, vp]
        _lib.or_cpml_profile.argtypes = [i, d, i, d, d, d, d, vp, vp, vp]
        _lib.or_cpml_profile.restype = None
        _lib.or_gaussian.argtypes = [d, i, vp, i]
        _lib.or_trapezoid.argtypes = [d, d, d, d, vp, i]
        _lib.or_moment_psv.argtypes = [d, d, d, d, vp]
        _lib.or_moment_psv.restype = None
        _lib.or_moment_sh.argtypes = [d, d, d, d, vp]
        _lib.or_moment_sh.restype = None
        _lib.or_psv_source_terms.argtypes = [i, i, i, i, vp, d, d, vp, i, i, vp, vp, vp]
        _lib.or_sh_source_terms.argtypes = [i, i, i, i, vp, d, d, vp, i, i, vp, vp, vp]
        _lib.or_mdl_raster.argtypes = [i, i, d, i, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        _lib.or_mdl_raster.restype = None
        for nm in ("or_psv_run_f64", "or_psv_run_f32", "or_psv_run_f32nf"):
            getattr(_lib, nm).argtypes = [i, i, i, i, vp, vp, i, vp, vp, vp, i, i, vp, i, vp,
                                          i, i, i, vp, vp, vp, i]
        for nm in ("or_sh_run_f64", "or_sh_run_f32", "or_sh_run_f32nf"):
            getattr(_lib, nm).argtypes = [i, i, i, i, vp, vp, i, vp, vp, vp, i, i, vp,
                                          i, i, i, vp, vp, i]
        _lib.or_set_punch.argtypes = [vp, vp, i]
        _lib.or_set_punch.restype = None
        _lib.or_box_ring_count.argtypes = [i, i, vp, vp]
        _lib.or_box_rings.argtypes = [i, i, i, i, i, vp, vp, vp, vp]
        _lib.or_box_incident_from_displacement.argtypes = [i, i, d, vp, vp, vp, vp, vp, vp]
        _lib.or_box_material.argtypes = [i, i, vp, i, i, i, i, d, d, d, d, d, vp]
        _lib.or_box_residual_step_f64.argtypes = [i, i, vp, vp]
        for nm in ("or_psv_box_run_f64", "or_psv_box_run_f32"):
            getattr(_lib, nm).argtypes = [i, i, i, i, vp, vp, i, vp, vp, vp, i, i, vp, vp,
                                          i, i, i, vp, vp, i, i, i, i, vp, vp, vp, i]
        _lib.or_line_source_coefs.argtypes = [d, d, d, d, vp]
        _lib.or_line_source_coefs.restype = None
        _lib.or_line_source_planes.argtypes = [i, i, i, i, d, d, d, d, d, vp, d, d, vp, i, i, i, vp]
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


# --------------------------------------------------------------------------
# model input
# --------------------------------------------------------------------------
def parse_mdl(path):
    """Parse a ``.mdl`` polygon model (BACK / POLY / DEF keywords), following
    the grammar read by PD/model/model.cpp:240-369.  Returns a list of
    (vp, vs, den, [(x, z), ...]) with the background first."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    polys, defs = [], {}
    k = 0
    while k < len(lines):
        line = lines[k]
        k += 1
        if not line.strip() or line.startswith("#"):
            continue
        args = line.split()
        key = args[0].upper()
        if key == "DEF":
            defs[args[1]] = (float(args[2]), float(args[3]))
            continue
        if key in ("BACK", "POLY"):
            vp, vs, den = (float(a) for a in args[1:4])
            if vs < 0:
                vs = -vp * vs
            if den < 0:
                den = -vp * den
            verts = []
            if key == "POLY":
                while k < len(lines) and lines[k].startswith("\t"):
                    toks = lines[k].split()
                    k += 1
                    j = 0
                    while j < len(toks):
                        if toks[0][0].isalpha():
                            verts.append(defs[toks[j]])
                            j += 1
                        else:
                            verts.append((float(toks[j]), float(toks[j + 1])))
                            j += 2
                polys.append((vp, vs, den, verts))
            else:
                polys.insert(0, (vp, vs, den, []))
            continue
        raise ValueError("bad model command %r" % line)
    return polys


def mdl_raster(polys, nx, nz, h):
    nvert = np.array([len(p[3]) for p in polys], dtype=np.int32)
    vx = np.array([v[0] for p in polys for v in p[3]] + [0.0], dtype=np.float64)
    vz = np.array([v[1] for p in polys for v in p[3]] + [0.0], dtype=np.float64)
    pvp = np.array([p[0] for p in polys], dtype=np.float64)
    pvs = np.array([p[1] for p in polys], dtype=np.float64)
    pden = np.array([p[2] for p in polys], dtype=np.float64)
    out = [np.empty(nx * nz, dtype=np.float64) for _ in range(3)]
    lib().or_mdl_raster(nx, nz, h, len(polys), _p(nvert), _p(vx), _p(vz), _p(pvp), _p(pvs),
                        _p(pden), _p(out[0]), _p(out[1]), _p(out[2]))
    return [o.reshape(nz, nx) for o in out]


# --------------------------------------------------------------------------
# material / CPML / source / receivers
# --------------------------------------------------------------------------
def psv_material(vp, vs, den, h, dt):
    nz, nx = vp.shape
    out = np.empty(5 * nx * nz, dtype=np.float64)
    stab = C.c_double(0.0)
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (vp, vs, den)]
    rc = lib().or_psv_material(nx, nz, h, dt, _p(a[0]), _p(a[1]), _p(a[2]), _p(out),
                               C.cast(C.pointer(stab), C.c_void_p))
    return out.reshape(5, nz, nx), stab.value, rc


def sh_material(vs, den, h, dt):
    nz, nx = vs.shape
    out = np.empty(3 * nx * nz, dtype=np.float64)
    stab = C.c_double(0.0)
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (vs, den)]
    rc = lib().or_sh_material(nx, nz, h, dt, _p(a[0]), _p(a[1]), _p(out),
                              C.cast(C.pointer(stab), C.c_void_p))
    return out.reshape(3, nz, nx), stab.value, rc


def cpml_profile(npml, startpos, n, pml_dt, pml_r, pml_v, pml_fc):
    b, c, k = (np.empty(n, dtype=np.float64) for _ in range(3))
    lib().or_cpml_profile(npml, startpos, n, pml_dt, pml_r, pml_v, pml_fc, _p(b), _p(c), _p(k))
    return b, c, k


def cpml_psv(nx, nz, npml, pml_dt, pml_r, pml_v, pml_fc):
    """b|c|k blocks; each block = Txx_x, Txz_x, U_x, W_x (nx) then
    Tzz_z, Txz_z, U_z, W_z (nz).  Start offsets from PD/cpml/cpml.cpp:177-185."""
    xs = [0.5, 0.0, 0.0, 0.5]  # Txx_x, Txz_x, U_x, W_x
    zs = [0.0, 0.5, 0.0, 0.5]  # Tzz_z, Txz_z, U_z, W_z
    out = np.empty((3, 4 * nx + 4 * nz), dtype=np.float64)
    for j, s in enumerate(xs):
        b, c, k = cpml_profile(npml, s, nx, pml_dt, pml_r, pml_v, pml_fc)
        for q, arr in enumerate((b, c, k)):
            out[q, j * nx:(j + 1) * nx] = arr
    for j, s in enumerate(zs):
        b, c, k = cpml_profile(npml, s, nz, pml_dt, pml_r, pml_v, pml_fc)
        for q, arr in enumerate((b, c, k)):
            out[q, 4 * nx + j * nz:4 * nx + (j + 1) * nz] = arr
    return out


def cpml_sh(nx, nz, npml, pml_dt, pml_r, pml_v, pml_fc):
    """b|c|k blocks; each block = Tx_x, V_x (nx) then Tz_z, V_z (nz).
    Start offsets from SH/cpml/cpml.cpp:172-176."""
    out = np.empty((3, 2 * nx + 2 * nz), dtype=np.float64)
    for j, (s, n, off) in enumerate(((0.0, nx, 0), (0.5, nx, nx), (0.5, nz, 2 * nx),
                                     (0.0, nz, 2 * nx + nz))):
        b, c, k = cpml_profile(npml, s, n, pml_dt, pml_r, pml_v, pml_fc)
        for q, arr in enumerate((b, c, k)):
            out[q, off:off + n] = arr
    return out


def gaussian(dt, alpha):
    cap = 2 * abs(int(alpha * 3.0)) + 2
    src = np.zeros(cap, dtype=np.float64)
    n = lib().or_gaussian(dt, int(alpha), _p(src), cap)
    return src[:n].copy()


def trapezoid(dt, t1, t2, t3):
    cap = int(t1 / dt) + int(t2 / dt) + int(t3 / dt) + 2
    src = np.zeros(cap, dtype=np.float64)
    n = lib().or_trapezoid(dt, t1, t2, t3, _p(src), cap)
    return src[:n].copy()


def ricker(dt, f0, t0=None):
    """Ricker wavelet sampled as s(t)*dt (the integral form the reference uses
    for its wavelets).  Not part of the reference; t0 defaults to 1.2/f0 and
    the length to round(2*t0/dt)+1 samples."""
    if t0 is None:
        t0 = 1.2 / f0
    n = int(round(2.0 * t0 / dt)) + 1
    t = np.arange(n, dtype=np.float64) * dt - t0
    a = (math.pi * f0 * t) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a) * dt


def moment_psv(strike, dip, rake, azimuth):
    m = np.empty(3, dtype=np.float64)
    lib().or_moment_psv(strike, dip, rake, azimuth, _p(m))
    return m


def moment_sh(strike, dip, rake, azimuth):
    m = np.empty(2, dtype=np.float64)
    lib().or_moment_sh(strike, dip, rake, azimuth, _p(m))
    return m


PSV_FIELDS = {"U": 0, "W": 1, "Txx": 2, "Txz": 3, "Tzz": 4}
SH_FIELDS = {"V": 0, "Tx": 1, "Tz": 2}


def source_terms(wave, kind, nx, xs, zs, moment, h, dt, src, nt):
    """Returns (field ids int32, flat cell idx int64, amp float64 [nterms, nt])."""
    src = np.ascontiguousarray(src, dtype=np.float64)
    field = np.zeros(16, dtype=np.int32)
    idx = np.zeros(16, dtype=np.int64)
    amp = np.zeros((16, nt), dtype=np.float64)
    m = np.ascontiguousarray(moment, dtype=np.float64)
    fn = lib().or_psv_source_terms if wave == "psv" else lib().or_sh_source_terms
    n = fn(kind, nx, xs, zs, _p(m), h, dt, _p(src), len(src), nt, _p(field), _p(idx), _p(amp))
    return field[:n].copy(), idx[:n].copy(), np.ascontiguousarray(amp[:n])


def receivers_line(nrec, ix0, iz0, idx, idz):
    """PD/record/cu_record.cu:12-28: each receiver is recorded as the pair
    (x, z), (x-1, z)."""
    rx, rz = [], []
    for i in range(nrec):
        x, z = ix0 + idx * i, iz0 + idz * i
        rx += [x, x - 1]
        rz += [z, z]
    return np.array(rx, dtype=np.int64), np.array(rz, dtype=np.int64)


def receivers_file(path):
    """Station file of (z x) pairs, PD/record/cu_record.cu:30-76."""
    vals = [int(t) for t in open(path).read().split()]
    rx, rz = [], []
    for j in range(0, len(vals) - 1, 2):
        z, x = vals[j], vals[j + 1]
        rx += [x, x - 1]
        rz += [z, z]
    return np.array(rx, dtype=np.int64), np.array(rz, dtype=np.int64)


# --------------------------------------------------------------------------
# time stepping
# --------------------------------------------------------------------------
def psv_state_size(nx, nz, npml):
    return 5 * nx * nz + 4 * 2 * npml * nz + 4 * 2 * npml * nx


def sh_state_size(nx, nz, npml):
    return 3 * nx * nz + 2 * 2 * npml * nz + 2 * 2 * npml * nx


class _Punch:
    """Installs tile step windows (first, last) in the C oracle for the
    duration of a run (None: no windows)."""

    def __init__(self, nx, punch):
        self.w = None
        if punch is not None:
            f, l = punch
            self.w = (np.ascontiguousarray(f, dtype=np.int32), np.ascontiguousarray(l, dtype=np.int32))
            self.nbx = (nx + 31) // 32

    def __enter__(self):
        if self.w is not None:
            lib().or_set_punch(_p(self.w[0]), _p(self.w[1]), self.nbx)

    def __exit__(self, *a):
        lib().or_set_punch(None, None, 0)


def psv_run(prec, nx, nz, npml, topabsorb, mat, bck, terms, rec_u, rec_w, nt, itrecord=1, it0=0,
            state=None, nthreads=0, punch=None):
    """Run nt steps of the P-SV oracle.  prec 'f64', 'f32' or 'f32nf' (FP32
    with every multiply-add rounded twice, no fused multiply-add).  mat (5,nz,nx)
    and bck (3, 4nx+4nz) FP64 arrays are rounded to prec.  terms = (field,
    idx, amp[nterms, nt_amp]) with absolute step indexing.  rec_* = flat
    indices.  punch = tile step windows (first, last), [nbz*nbx] each, or
    None.  Returns (seis_u, seis_w, state)."""
    dt_ = np.float64 if prec == "f64" else np.float32
    fn = getattr(lib(), "or_psv_run_" + prec)
    mat_r = np.ascontiguousarray(mat, dtype=dt_)
    bck_r = np.ascontiguousarray(bck, dtype=dt_)
    field, idx, amp = terms
    field = np.ascontiguousarray(field, dtype=np.int32)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    amp_r = np.ascontiguousarray(amp, dtype=dt_)
    ru = np.ascontiguousarray(rec_u, dtype=np.int64)
    rw = np.ascontiguousarray(rec_w, dtype=np.int64)
    if state is None:
        state = np.zeros(psv_state_size(nx, nz, npml), dtype=dt_)
    else:
        state = np.ascontiguousarray(state, dtype=dt_).copy()
    nrecs = len([it for it in range(it0, it0 + nt) if it % itrecord == 0])
    su = np.zeros((nrecs, len(ru)), dtype=dt_)
    sw = np.zeros((nrecs, len(rw)), dtype=dt_)
    nt_amp = amp_r.shape[1] if amp_r.ndim == 2 and len(field) else 0
    with _Punch(nx, punch):
        fn(nx, nz, npml, int(topabsorb), _p(mat_r), _p(bck_r), len(field), _p(field), _p(idx),
           _p(amp_r) if len(field) else None, nt_amp, len(ru), _p(ru), len(rw), _p(rw), it0, nt,
           itrecord, _p(state), _p(su), _p(sw), nthreads)
    return su, sw, state


def sh_run(prec, nx, nz, npml, topabsorb, mat, bck, terms, rec, nt, itrecord=1, it0=0, state=None,
           nthreads=0, punch=None):
    dt_ = np.float64 if prec == "f64" else np.float32
    fn = getattr(lib(), "or_sh_run_" + prec)
    mat_r = np.ascontiguousarray(mat, dtype=dt_)
    bck_r = np.ascontiguousarray(bck, dtype=dt_)
    field, idx, amp = terms
    field = np.ascontiguousarray(field, dtype=np.int32)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    amp_r = np.ascontiguousarray(amp, dtype=dt_)
    r = np.ascontiguousarray(rec, dtype=np.int64)
    if state is None:
        state = np.zeros(sh_state_size(nx, nz, npml), dtype=dt_)
    else:
        state = np.ascontiguousarray(state, dtype=dt_).copy()
    nrecs = len([it for it in range(it0, it0 + nt) if it % itrecord == 0])
    s = np.zeros((nrecs, len(r)), dtype=dt_)
    nt_amp = amp_r.shape[1] if amp_r.ndim == 2 and len(field) else 0
    with _Punch(nx, punch):
        fn(nx, nz, npml, int(topabsorb), _p(mat_r), _p(bck_r), len(field), _p(field), _p(idx),
           _p(amp_r) if len(field) else None, nt_amp, len(r), _p(r), it0, nt, itrecord, _p(state),
           _p(s), nthreads)
    return s, state


def punch_windows(times, before, after, dt, elem="f64"):
    """Tile step windows from travel times t[nz, nx], restating the SLIDE
    constructor (PD/slide/cu_slide.cu:23-55): over tiles of 32 columns x 16
    rows, first = int((tmin - before)/dt), last = int((tmax + after)/dt).
    elem 'f64': double times and arithmetic (PD); 'f32': float (PN/SH,
    PN/slide/cu_slide.cu:10-12).  min/max start from +/-1e28 and skip NaN;
    edge tiles of grids that are not whole tiles cover the cells they have;
    the int conversion truncates and saturates (NaN gives 0).
    Returns (first, last), int32 [nbz*nbx]."""
    T = np.float64 if elem == "f64" else np.float32
    t = np.asarray(times, dtype=T)
    nz, nx = t.shape
    nbx, nbz = (nx + 31) // 32, (nz + 15) // 16
    lo = np.full((nbz * 16, nbx * 32), np.inf, dtype=T)
    hi = np.full((nbz * 16, nbx * 32), -np.inf, dtype=T)
    lo[:nz, :nx] = t
    hi[:nz, :nx] = t
    lo = np.fmin.reduce(np.fmin.reduce(lo.reshape(nbz, 16, nbx, 32), axis=3), axis=1)
    hi = np.fmax.reduce(np.fmax.reduce(hi.reshape(nbz, 16, nbx, 32), axis=3), axis=1)
    lo = np.fmin(lo, T(1e28))
    hi = np.fmax(hi, T(-1e28))
    with np.errstate(all="ignore"):
        a = (lo - T(before)) / T(dt)
        b = (hi + T(after)) / T(dt)

    def to_int(v):
        v = v.astype(np.float64)  # exact for float32 and for the comparisons
        out = np.where(np.isnan(v), 0.0, np.trunc(v))
        out = np.clip(out, -2147483648.0, 2147483647.0)
        return out.astype(np.int64).astype(np.int32).ravel()

    return to_int(a), to_int(b)


# ---------------------------------------------------------------- hybrid box
def box_ring_count(bx, bz):
    """(nsub, nadd) ring sizes of a bx x bz box (PD/box/box.cpp:59-95)."""
    ns = np.zeros(1, np.int32)
    na = np.zeros(1, np.int32)
    if lib().or_box_ring_count(bx, bz, _p(ns), _p(na)) < 0:
        raise ValueError("box must be at least 16 x 16")
    return int(ns[0]), int(na[0])


def box_rings(nx, x0, z0, bx, bz):
    """Ring cells in incident-field order: (grid flat index, box flat index,
    nsub)."""
    nsub, nadd = box_ring_count(bx, bz)
    g = np.zeros(nsub + nadd, np.int64)
    r = np.zeros(nsub + nadd, np.int64)
    ns = np.zeros(1, np.int32)
    na = np.zeros(1, np.int32)
    lib().or_box_rings(nx, x0, z0, bx, bz, _p(g), _p(r), _p(ns), _p(na))
    return g, r, nsub


def box_incident_from_displacement(bx, bz, dt, rmat, uo, wo, un, wn):
    """BOX::setboxsource restated (PD/box/box.cpp:120-196): ring incident
    field [5, nring] from displacement planes of shape (bz+8, bx+8)."""
    nsub, nadd = box_ring_count(bx, bz)
    out = np.zeros((5, nsub + nadd))
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (rmat, uo, wo, un, wn)]
    lib().or_box_incident_from_displacement(bx, bz, dt, *[_p(v) for v in a], _p(out))
    return out


def line_source_coefs(strike, dip, rake, azimuth):
    """Radiation coefficients (A1, A2, A3) of the line moment source
    (PD/source/source_line.cpp:320-326)."""
    a = np.zeros(3)
    lib().or_line_source_coefs(strike, dip, rake, azimuth, _p(a))
    return a


def box_plane_origin(bw):
    """Source-relative cell offset of plane cell (0, 0) for the reference's
    square box of width bw (PD/source/source_line.cpp:346-347)."""
    return (bw + 1) // 2 + 4 + 1 - (bw + 8)


def line_source_planes(px, pz, ox, oz, h, dt, vp, vs, den, a, src, it0, nf, sx=0.25, sz=-0.25):
    """Displacement planes of the box-source generator (ntde_line,
    PD/source/source_line.cpp:307-410): array [nf, 2, pz, px] of frames
    it0 .. it0+nf-1 (U plane, W plane), the layout of the reference's source
    file."""
    out = np.zeros((nf, 2, pz, px))
    src = np.ascontiguousarray(src, dtype=np.float64)
    a = np.ascontiguousarray(a, dtype=np.float64)
    rc = lib().or_line_source_planes(px, pz, ox, oz, h, dt, vp, vs, den, _p(a), sx, sz, _p(src), len(src),
                                     it0, nf, _p(out))
    if rc:
        raise ValueError("bad line-source arguments")
    return out


def box_material(mat, x0, z0, bx, bz, srcvp, srcvs, srcden, dt, h):
    """MATERIAL::init_for_box_from_full restated (PD/material/material.cpp:39-97).
    Returns (full material with the box homogenised, box material, cells
    replaced)."""
    m = np.ascontiguousarray(mat, dtype=np.float64).copy()
    nz, nx = m.shape[1], m.shape[2]
    rm = np.zeros((5, bz, bx))
    n = lib().or_box_material(nx, nz, _p(m), x0, z0, bx, bz, srcvp, srcvs, srcden, dt, h, _p(rm))
    return m, rm, n


def psv_box_run(prec, nx, nz, npml, topabsorb, mat, bck, terms, rec_field, rec_idx, nt, box, rmat,
                inc, itrecord=1, it0=0, state=None, rstate=None, nthreads=0):
    """Hybrid-box P-SV run.  box = (x0, z0, bx, bz); rmat (5, bz, bx); inc
    [nt, 5, nring] for steps it0 .. it0+nt-1; receivers are (field, flat
    index) pairs.  Returns (seis [nrec_steps, nrec], state, rstate)."""
    dt_ = np.float64 if prec == "f64" else np.float32
    fn = lib().or_psv_box_run_f64 if prec == "f64" else lib().or_psv_box_run_f32
    x0, z0, bx, bz = box
    mat_r = np.ascontiguousarray(mat, dtype=dt_)
    bck_r = np.ascontiguousarray(bck, dtype=dt_)
    field, idx, amp = terms
    field = np.ascontiguousarray(field, dtype=np.int32)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    amp_r = np.ascontiguousarray(amp, dtype=dt_)
    rf = np.ascontiguousarray(rec_field, dtype=np.int32)
    ri = np.ascontiguousarray(rec_idx, dtype=np.int64)
    state = (np.zeros(psv_state_size(nx, nz, npml), dtype=dt_) if state is None
             else np.ascontiguousarray(state, dtype=dt_).copy())
    rstate = (np.zeros(5 * bx * bz, dtype=dt_) if rstate is None
              else np.ascontiguousarray(rstate, dtype=dt_).copy())
    rmat_r = np.ascontiguousarray(rmat, dtype=dt_)
    inc_r = np.ascontiguousarray(inc, dtype=dt_)
    nrecs = len([it for it in range(it0, it0 + nt) if it % itrecord == 0])
    seis = np.zeros((nrecs, len(rf)), dtype=dt_)
    nt_amp = amp_r.shape[1] if amp_r.ndim == 2 and len(field) else 0
    rc = fn(nx, nz, npml, int(topabsorb), _p(mat_r), _p(bck_r), len(field), _p(field), _p(idx),
            _p(amp_r) if len(field) else None, nt_amp, len(rf), _p(rf), _p(ri), it0, nt, itrecord,
            _p(state), _p(seis), x0, z0, bx, bz, _p(rmat_r), _p(rstate), _p(inc_r), nthreads)
    if rc < 0:
        raise ValueError("bad box")
    return seis, state, rstate


def box_residual_step(rmat, r):
    """One residual step (stress then velocity) of a box residual field
    r = [U W Txx Txz Tzz] of shape (5, bz, bx) in the box material rmat
    (5, bz, bx), FP64: the update the box run applies between its ring
    exchanges (PD/fd/fd.cpp:63-91, 208-234).  Returns the new field."""
    rm = np.ascontiguousarray(rmat, dtype=np.float64)
    out = np.ascontiguousarray(r, dtype=np.float64).copy()
    bz, bx = out.shape[1], out.shape[2]
    lib().or_box_residual_step_f64(bx, bz, _p(rm), _p(out))
    return out


def psv_ring_history(prec, nx, nz, npml, topabsorb, mat, bck, terms, nt, box, it0=0, state=None):
    """Run the plain P-SV oracle step by step and collect, for each step it,
    the incident field a box driven by this run needs: U, W before the step
    and Txx, Txz, Tzz after its stress update and source, on the ring cells.
    Returns (inc [nt, 5, nring], final state)."""
    x0, z0, bx, bz = box
    g, _, _ = box_rings(nx, x0, z0, bx, bz)
    n = nx * nz
    dt_ = np.float64 if prec == "f64" else np.float32
    st = (np.zeros(psv_state_size(nx, nz, npml), dtype=dt_) if state is None
          else np.asarray(state, dtype=dt_).copy())
    inc = np.zeros((nt, 5, len(g)), dtype=dt_)
    for k in range(nt):
        inc[k, 0] = st[g]
        inc[k, 1] = st[n + g]
        _, _, st = psv_run(prec, nx, nz, npml, topabsorb, mat, bck, terms, [], [], 1, 1,
                           it0=it0 + k, state=st)
        for f in range(2, 5):
            inc[k, f] = st[f * n + g]
    return inc, st


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
