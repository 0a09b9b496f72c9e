"""fd23_gb300 -- GB300 (sm_103a) 2-D elastic time stepping (P-SV and SH).

Python front end of the C ABI in include/fd23.h.  The compute path is the
CUDA library fd23_gb300/_lib/libfd23.so (build it with
``python -c "import fd23_gb300.build as b; b.build()"``); there is no CPU
fallback and importing this package without the library raises.

The objects mirror the operator surface of the reference fd23 programs
(paths relative to the fd23 project root):

  Solver(...)                PARAM + FIELD + CPML set-up (PD/param/param.cpp,
                             PD/field/cu_field.cu, PD/cpml/cpml.cpp)
  Solver.set_model           MATERIAL::get_model (PD/material/material.cpp:101)
  Solver.set_source          gaussian/trapozoid + cu_point_source(_p)
                             (PD/source/waveform.cpp, PD/point_source/)
  Solver.set_receivers       RECORD::init_line / init_list (PD/record/cu_record.cu)
  Solver.run                 the time loop of PN/main.cpp:117-170
  Solver.seismograms         the <output>_U / _W records ([step][receiver])
  Solver.get_state/set_state savestate / restart (PN/main.cpp:253-317)
"""
import ctypes as _C
import os as _os

import numpy as _np

_HERE = _os.path.dirname(_os.path.abspath(__file__))
LIB_PATH = _os.environ.get("FD23_LIB") or _os.path.join(_HERE, "_lib", "libfd23.so")

PSV, SH = 0, 1
F32, F64, BF16, F16 = 0, 1, 2, 3
KERNEL_AUTO, KERNEL_FUSED, KERNEL_TWOPASS, KERNEL_PERSIST, KERNEL_FUSED2 = 0, 1, 2, 3, 4
U, W, TXX, TXZ, TZZ = 0, 1, 2, 3, 4
V, TX, TZ = 0, 1, 2
SRC_EXPLOSION, SRC_FORCE, SRC_MOMENT, SRC_MOMENT_P = 1, 2, 3, 13
OK, ERR_ARG, ERR_CUDA, ERR_UNSTABLE, ERR_ORDER, ERR_NOMEM, ERR_NONFINITE, ERR_TIMEOUT, \
    ERR_UNSUPPORTED = 0, -1, -2, -3, -4, -5, -6, -7, -8

_WAVES = {"psv": PSV, "sh": SH, PSV: PSV, SH: SH}
_PRECS = {"f32": F32, "fp32": F32, "f64": F64, "fp64": F64, "bf16": BF16, "f16": F16,
          "fp16": F16, F32: F32, F64: F64, BF16: BF16, F16: F16}
_KERNELS = {"auto": KERNEL_AUTO, "fused": KERNEL_FUSED, "twopass": KERNEL_TWOPASS, "persist": KERNEL_PERSIST,
            "fused2": KERNEL_FUSED2, KERNEL_AUTO: KERNEL_AUTO, KERNEL_FUSED: KERNEL_FUSED,
            KERNEL_TWOPASS: KERNEL_TWOPASS, KERNEL_PERSIST: KERNEL_PERSIST, KERNEL_FUSED2: KERNEL_FUSED2}

# every function the C ABI exports (checked against include/fd23.h by the tests)
ABI_FUNCTIONS = [
    "fd23_create", "fd23_destroy", "fd23_strerror", "fd23_version", "fd23_set_model",
    "fd23_set_material", "fd23_set_cpml", "fd23_set_source", "fd23_set_source_terms",
    "fd23_wavelet_gaussian", "fd23_wavelet_trapezoid", "fd23_wavelet_ricker", "fd23_moment_psv",
    "fd23_moment_sh", "fd23_set_receivers", "fd23_receivers_line", "fd23_run", "fd23_sync",
    "fd23_get_seismograms", "fd23_reset", "fd23_get_stream", "fd23_get_step", "fd23_get_field_device", "fd23_state_bytes", "fd23_get_state",
    "fd23_set_state", "fd23_field_norm2", "fd23_build_material", "fd23_build_cpml",
    "fd23_build_source_terms", "fd23_sum_squares_noalloc", "fd23_set_box", "fd23_set_box_incident",
    "fd23_set_box_incident_async", "fd23_set_model_box",
    "fd23_box_state_bytes", "fd23_get_box_state", "fd23_set_box_state", "fd23_box_ring_size",
    "fd23_box_ring_index", "fd23_box_ring_cells", "fd23_box_incident_from_displacement",
    "fd23_box_material", "fd23_batch_create", "fd23_batch_destroy", "fd23_batch_run", "fd23_batch_sync",
    "fd23_batch_get_stream", "fd23_batch_set_graph", "fd23_autotune", "fd23_batch_autotune",
    "fd23_batch_get_plan", "fd23_batch_set_plan", "fd23_work_plan", "fd23_read_model", "fd23_read_stations",
    "fd23_debug_expire_wait", "fd23_set_plan", "fd23_get_plan", "fd23_punch_tiles", "fd23_punch_windows", "fd23_read_punch", "fd23_set_punch",
    "fd23_set_material_table", "fd23_set_punch_phase", "fd23_work_plan_live",
    "fd23_line_source_coefs", "fd23_line_plane_origin", "fd23_line_source_planes", "fd23_set_box_line_source",
    "fd23_debug_persist_barrier",
]


class Fd23Error(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        msg = lib().fd23_strerror(status).decode() if _lib is not None else str(status)
        super().__init__("%s: %s (status %d)" % (where, msg, status))


class TuneEntry(_C.Structure):
    _fields_ = [("wx", _C.c_double), ("wz", _C.c_double), ("per_sm", _C.c_int), ("bands", _C.c_int),
                ("oversub", _C.c_double), ("ms_per_step", _C.c_double), ("fast_iter", _C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LineDesc(_C.Structure):
    """fd23_line_desc: planes of the box-source generator."""
    _fields_ = [("px", _C.c_int), ("pz", _C.c_int), ("ox", _C.c_int), ("oz", _C.c_int),
                ("h", _C.c_double), ("dt", _C.c_double), ("vp", _C.c_double), ("vs", _C.c_double),
                ("den", _C.c_double), ("a", _C.c_double * 3), ("sx", _C.c_double), ("sz", _C.c_double)]


def line_desc(px, pz, ox, oz, h, dt, vp, vs, den, a, sx=0.25, sz=-0.25):
    """A LineDesc; a = line_source_coefs(strike, dip, rake, azimuth)."""
    return LineDesc(px, pz, ox, oz, h, dt, vp, vs, den, (_C.c_double * 3)(*[float(v) for v in a]), sx, sz)


class Desc(_C.Structure):
    _fields_ = [("wave", _C.c_int), ("prec", _C.c_int), ("nx", _C.c_int), ("nz", _C.c_int),
                ("npml", _C.c_int), ("topabsorb", _C.c_int), ("h", _C.c_double),
                ("dt", _C.c_double), ("pml_dt", _C.c_double), ("pml_v", _C.c_double),
                ("pml_r", _C.c_double), ("pml_fc", _C.c_double), ("device", _C.c_int),
                ("kernel", _C.c_int)]


_lib = None


def lib():
    """Load libfd23.so (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not _os.path.exists(LIB_PATH):
        raise ImportError("fd23 CUDA library not built: %s is missing (run fd23_gb300/build.py)"
                          % LIB_PATH)
    L = _C.CDLL(LIB_PATH)
    vp, i, d, sz = _C.c_void_p, _C.c_int, _C.c_double, _C.c_size_t
    sig = {
        "fd23_create": ([_C.POINTER(Desc), _C.POINTER(vp)], i),
        "fd23_destroy": ([vp], None),
        "fd23_strerror": ([i], _C.c_char_p),
        "fd23_version": ([], i),
        "fd23_set_model": ([vp, vp, vp, vp, vp], i),
        "fd23_set_material": ([vp, vp], i),
        "fd23_set_cpml": ([vp, vp], i),
        "fd23_set_source": ([vp, i, i, i, vp, vp, i, i], i),
        "fd23_set_source_terms": ([vp, i, vp, vp, vp, vp, i], i),
        "fd23_wavelet_gaussian": ([d, i, vp, i], i),
        "fd23_wavelet_trapezoid": ([d, d, d, d, vp, i], i),
        "fd23_wavelet_ricker": ([d, d, d, vp, i], i),
        "fd23_moment_psv": ([d, d, d, d, vp], None),
        "fd23_moment_sh": ([d, d, d, d, vp], None),
        "fd23_set_receivers": ([vp, i, vp, vp, i], i),
        "fd23_receivers_line": ([i, i, i, i, i, vp, vp], i),
        "fd23_run": ([vp, i, i], i),
        "fd23_sync": ([vp], i),
        "fd23_get_seismograms": ([vp, i, vp, sz, _C.POINTER(i)], i),
        "fd23_reset": ([vp], i),
        "fd23_get_stream": ([vp, _C.POINTER(vp)], i),
        "fd23_get_step": ([vp, _C.POINTER(i)], i),
        "fd23_get_field_device": ([vp, i, _C.POINTER(vp), _C.POINTER(sz)], i),
        "fd23_state_bytes": ([vp], sz),
        "fd23_get_state": ([vp, vp, sz], i),
        "fd23_set_state": ([vp, vp, sz, i], i),
        "fd23_field_norm2": ([vp, _C.POINTER(d)], i),
        "fd23_build_material": ([i, i, i, d, d, vp, vp, vp, vp, vp], i),
        "fd23_build_cpml": ([i, i, i, i, d, d, d, d, vp, sz], i),
        "fd23_build_source_terms": ([i, i, i, i, vp, d, d, vp, i, i, vp, vp, vp, vp, i], i),
        "fd23_sum_squares_noalloc": ([i, vp, i, sz, vp, _C.POINTER(d), _C.POINTER(i)], i),
        "fd23_set_box": ([vp, i, i, i, i, vp], i),
        "fd23_set_model_box": ([vp, vp, vp, vp, i, i, i, i, d, d, d, vp, vp, vp], i),
        "fd23_set_box_incident": ([vp, vp, i, i], i),
        "fd23_set_box_incident_async": ([vp, vp, i, i], i),
        "fd23_box_state_bytes": ([vp], sz),
        "fd23_get_box_state": ([vp, vp, sz], i),
        "fd23_set_box_state": ([vp, vp, sz], i),
        "fd23_box_ring_size": ([i, i, _C.POINTER(i), _C.POINTER(i)], i),
        "fd23_box_ring_index": ([i, i, i, i], i),
        "fd23_box_ring_cells": ([i, i, i, i, vp, vp], i),
        "fd23_box_incident_from_displacement": ([i, i, d, vp, vp, vp, vp, vp, vp], i),
        "fd23_box_material": ([i, i, vp, i, i, i, i, d, d, d, d, d, vp], i),
        "fd23_batch_create": ([vp, i, _C.POINTER(vp)], i),
        "fd23_batch_destroy": ([vp], None),
        "fd23_batch_run": ([vp, i, i], i),
        "fd23_batch_sync": ([vp], i),
        "fd23_batch_get_stream": ([vp, _C.POINTER(vp)], i),
        "fd23_batch_set_graph": ([vp, i], i),
        "fd23_batch_set_plan": ([vp, vp], i),
        "fd23_autotune": ([vp, i, vp, i], i),
        "fd23_batch_autotune": ([vp, i, vp, i], i),
        "fd23_batch_get_plan": ([vp, vp, _C.POINTER(i)], i),
        "fd23_work_plan": ([i, vp, vp, vp, vp, i, vp, vp, i, vp, i], i),
        "fd23_read_model": ([_C.c_char_p, i, i, d, vp, vp, vp], i),
        "fd23_read_stations": ([_C.c_char_p, vp, vp, i], i),
        "fd23_debug_expire_wait": ([vp], i),
        "fd23_debug_persist_barrier": ([vp], i),
        "fd23_set_plan": ([vp, vp], i),
        "fd23_get_plan": ([vp, vp, _C.POINTER(i)], i),
        "fd23_punch_tiles": ([i, i, _C.POINTER(i), _C.POINTER(i)], i),
        "fd23_punch_windows": ([vp, i, i, i, d, d, d, vp, vp], i),
        "fd23_read_punch": ([_C.c_char_p, i, i, i, d, d, d, vp, vp], i),
        "fd23_set_punch": ([vp, vp, vp, i, i], i),
        "fd23_set_material_table": ([vp, i], i),
        "fd23_set_punch_phase": ([vp, i], i),
        "fd23_work_plan_live": ([i, vp, vp, vp, vp, i, vp, vp, vp, i, vp, i], i),
        "fd23_line_source_coefs": ([d, d, d, d, vp], i),
        "fd23_line_plane_origin": ([i], i),
        "fd23_line_source_planes": ([i, _C.POINTER(LineDesc), vp, i, i, i, vp], i),
        "fd23_set_box_line_source": ([vp, _C.POINTER(LineDesc), vp, i, vp, i, i], i),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(_C.c_void_p)


def _f64(a):
    return _np.ascontiguousarray(a, dtype=_np.float64)


def _i32(a):
    return _np.ascontiguousarray(a, dtype=_np.int32)


def _sized(a, n, what):
    """a as a contiguous array of exactly n elements (the C side reads n)."""
    if a.size != n:
        raise ValueError("%s: %d elements, expected %d" % (what, a.size, n))
    return a


def _check(rc, where):
    if rc < 0:
        raise Fd23Error(rc, where)
    return rc


# ---------------------------------------------------------------------------
# host-side builders (no GPU needed)
def build_material(wave, vp, vs, den, h, dt):
    """FP64 staggered material, dt/h scaled.  Returns (mat[nmat, nz, nx], stab, status)."""
    w = _WAVES[wave]
    vs = _f64(vs)
    nz, nx = vs.shape
    nmat = 5 if w == PSV else 3
    out = _np.empty((nmat, nz, nx), dtype=_np.float64)
    stab = _C.c_double(0.0)
    rc = lib().fd23_build_material(w, nx, nz, h, dt, _p(_f64(vp)) if vp is not None else None,
                                   _p(vs), _p(_f64(den)), _p(out),
                                   _C.cast(_C.pointer(stab), _C.c_void_p))
    return out, stab.value, rc


def build_cpml(wave, nx, nz, npml, pml_dt, pml_r, pml_v, pml_fc):
    w = _WAVES[wave]
    n = 3 * ((8 if w == PSV else 4) // 2) * (nx + nz)
    out = _np.empty(n, dtype=_np.float64)
    k = _check(lib().fd23_build_cpml(w, nx, nz, npml, pml_dt, pml_r, pml_v, pml_fc, _p(out), n),
               "fd23_build_cpml")
    return out[:k].reshape(3, -1)


def wavelet_gaussian(dt, alpha):
    cap = 2 * abs(int(alpha * 3.0)) + 2
    out = _np.zeros(cap)
    n = _check(lib().fd23_wavelet_gaussian(dt, int(alpha), _p(out), cap), "gaussian")
    return out[:n].copy()


def wavelet_trapezoid(dt, t1, t2, t3):
    cap = int(t1 / dt) + int(t2 / dt) + int(t3 / dt) + 4
    out = _np.zeros(cap)
    n = _check(lib().fd23_wavelet_trapezoid(dt, t1, t2, t3, _p(out), cap), "trapezoid")
    return out[:n].copy()


def wavelet_ricker(dt, f0, t0=0.0):
    cap = int(round(2.0 * (t0 if t0 > 0 else 1.2 / f0) / dt)) + 4
    out = _np.zeros(cap)
    n = _check(lib().fd23_wavelet_ricker(dt, f0, t0, _p(out), cap), "ricker")
    return out[:n].copy()


def moment_psv(strike, dip, rake, azimuth):
    m = _np.zeros(3)
    lib().fd23_moment_psv(strike, dip, rake, azimuth, _p(m))
    return m


def moment_sh(strike, dip, rake, azimuth):
    m = _np.zeros(2)
    lib().fd23_moment_sh(strike, dip, rake, azimuth, _p(m))
    return m


def build_source_terms(wave, kind, xs, zs, moment, h, dt, src, nt):
    src = _f64(src)
    f, x, z = (_np.zeros(16, dtype=_np.int32) for _ in range(3))
    amp = _np.zeros((16, nt))
    m = _f64(moment) if moment is not None else _np.zeros(3)
    n = _check(lib().fd23_build_source_terms(_WAVES[wave], kind, xs, zs, _p(m), h, dt, _p(src),
                                             len(src), nt, _p(f), _p(x), _p(z), _p(amp), 16),
               "fd23_build_source_terms")
    return f[:n].copy(), x[:n].copy(), z[:n].copy(), _np.ascontiguousarray(amp[:n])


def sum_squares_noalloc(prec, field_ptrs, n, stream=0):
    """Allocation-free FP64 sum of squares of device arrays (raw device
    pointers, n elements each, element type prec); returns (sum, nonfinite).
    Callers that cannot allocate device memory use this instead of
    Solver.norm2; see include/fd23.h for its limits."""
    ptrs = (_C.c_void_p * max(1, len(field_ptrs)))(*[_C.c_void_p(int(p)) for p in field_ptrs])
    total = _C.c_double(0.0)
    bad = _C.c_int(0)
    _check(lib().fd23_sum_squares_noalloc(_PRECS[prec], _C.cast(ptrs, _C.c_void_p), len(field_ptrs), n,
                                          _C.c_void_p(int(stream)) if stream else None,
                                          _C.byref(total), _C.byref(bad)), "fd23_sum_squares_noalloc")
    return total.value, bool(bad.value)


# ---------------------------------------------------------------- hybrid box
def box_ring_size(bx, bz):
    """(nsub, nadd): cells of the sub ring (outer 4 of the box) and of the add
    ring (the next 4 inward)."""
    ns, na = _C.c_int(0), _C.c_int(0)
    _check(lib().fd23_box_ring_size(bx, bz, _C.byref(ns), _C.byref(na)), "fd23_box_ring_size")
    return ns.value, na.value


def box_ring_index(bx, bz, bi, bj):
    """Ring position of box cell (bi, bj), -1 when it is in neither ring."""
    return lib().fd23_box_ring_index(bx, bz, bi, bj)


def box_ring_cells(x0, z0, bx, bz):
    """Grid cells (ix, iz) of every ring position, in incident-field order."""
    n = sum(box_ring_size(bx, bz))
    ix = _np.zeros(n, _np.int32)
    iz = _np.zeros(n, _np.int32)
    _check(lib().fd23_box_ring_cells(x0, z0, bx, bz, _p(ix), _p(iz)), "fd23_box_ring_cells")
    return ix, iz


def box_incident_from_displacement(bx, bz, dt, bmat, u_old, w_old, u_new, w_new):
    """Incident field [5, nring] of one step from displacement planes of
    shape (bz+8, bx+8) (BOX::setboxsource)."""
    n = sum(box_ring_size(bx, bz))
    out = _np.zeros((5, n))
    a = [_f64(v) for v in (bmat, u_old, w_old, u_new, w_new)]
    _check(lib().fd23_box_incident_from_displacement(bx, bz, dt, *[_p(v) for v in a], _p(out)),
           "fd23_box_incident_from_displacement")
    return out


def line_source_coefs(strike, dip, rake, azimuth):
    """Radiation coefficients (A1, A2, A3) of the line moment source."""
    a = _np.zeros(3)
    _check(lib().fd23_line_source_coefs(strike, dip, rake, azimuth, _p(a)), "fd23_line_source_coefs")
    return a


def line_plane_origin(bw):
    """Source-relative offset of plane cell (0, 0) of the reference's
    bw x bw box."""
    return lib().fd23_line_plane_origin(bw)


def line_source_planes(desc, src, it0, nframes, device=0):
    """Frames it0 .. it0+nframes-1 of the box-source generator on the GPU:
    array [nframes, 2, pz, px] (U plane, W plane), the source-file layout."""
    src = _f64(src)
    out = _np.zeros((nframes, 2, desc.pz, desc.px))
    _check(lib().fd23_line_source_planes(device, _C.byref(desc), _p(src), len(src), it0, nframes, _p(out)),
           "fd23_line_source_planes")
    return out


def box_material(mat, x0, z0, bx, bz, src_vp, src_vs, src_den, dt, h):
    """(grid material with the box made homogeneous, box material (5, bz, bx),
    cells replaced): MATERIAL::init_for_box_from_full."""
    m = _f64(mat).copy()
    nz, nx = m.shape[-2], m.shape[-1]
    bm = _np.zeros((5, bz, bx))
    n = _check(lib().fd23_box_material(nx, nz, _p(m), x0, z0, bx, bz, src_vp, src_vs, src_den, dt, h,
                                       _p(bm)), "fd23_box_material")
    return m, bm, n


def work_plan(grids, sms=152, wx=4.0, wz=3.0, per_sm=3, oversub=1.0, live=None, bands=1):
    """The fused sweep's work plan for grids [(nx, nz, npml, topabsorb)]:
    list over CTAs of lists of (shot, x0, z0, z1) items.  live: optional
    per-grid boolean arrays over the 4-row blocks (strip-major) to plan;
    bands=1: every strip cut on its own (fd23_tune_entry.bands)."""
    n = len(grids)
    a = [_np.ascontiguousarray([g[k] for g in grids], dtype=_np.int32) for k in range(4)]
    cap = sum(((g[0] + 119) // 120) * ((g[1] + 3) // 4) for g in grids) * 2 + 16
    items = _np.zeros(4 * cap, _np.int32)
    off = _np.zeros(cap + 1, _np.int32)
    t = TuneEntry(wx=wx, wz=wz, per_sm=per_sm, bands=bands, oversub=oversub)
    lv = None if live is None else _np.ascontiguousarray(_np.concatenate([_np.asarray(m, bool).ravel()
                                                                           for m in live]), dtype=_np.uint8)
    nb = _check(lib().fd23_work_plan_live(n, *[_p(v) for v in a], sms, _C.cast(_C.pointer(t), _C.c_void_p),
                                          _p(lv), _p(items), cap, _p(off), cap), "fd23_work_plan_live")
    it = items.reshape(-1, 4)
    return [[tuple(int(v) for v in it[j]) for j in range(off[c], off[c + 1])] for c in range(nb)]


class Batch:
    """Several solvers advanced in lockstep, one sweep launch per step for all
    shots (CUDA-graph captured)."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        arr = (_C.c_void_p * len(self.solvers))(*[s._h.value for s in self.solvers])
        self._h = _C.c_void_p()
        _check(lib().fd23_batch_create(_C.cast(arr, _C.c_void_p), len(self.solvers), _C.byref(self._h)),
               "fd23_batch_create")

    def close(self):
        if self._h:
            lib().fd23_batch_destroy(self._h)
            self._h = _C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, nsteps, itrecord=1):
        _check(lib().fd23_batch_run(self._h, nsteps, itrecord), "fd23_batch_run")

    def sync(self):
        _check(lib().fd23_batch_sync(self._h), "fd23_batch_sync")

    @property
    def stream(self):
        p = _C.c_void_p()
        _check(lib().fd23_batch_get_stream(self._h, _C.byref(p)), "fd23_batch_get_stream")
        return p.value or 0

    def set_graph(self, on):
        _check(lib().fd23_batch_set_graph(self._h, int(bool(on))), "fd23_batch_set_graph")

    def plan(self):
        e = TuneEntry()
        nb = _C.c_int(0)
        _check(lib().fd23_batch_get_plan(self._h, _C.cast(_C.pointer(e), _C.c_void_p), _C.byref(nb)),
               "fd23_batch_get_plan")
        d = e.as_dict()
        d["nblocks"] = nb.value
        return d

    def set_plan(self, wx=4.0, wz=3.0, per_sm=3, oversub=1.0, bands=1):
        """Install a work plan for the batch without timing it (fd23_batch_set_plan)."""
        t = TuneEntry(wx=wx, wz=wz, per_sm=per_sm, bands=bands, oversub=oversub)
        _check(lib().fd23_batch_set_plan(self._h, _C.cast(_C.pointer(t), _C.c_void_p)), "fd23_batch_set_plan")

    def autotune(self, trial_steps=10):
        tab = (TuneEntry * 256)()
        n = _check(lib().fd23_batch_autotune(self._h, trial_steps, _C.cast(tab, _C.c_void_p), 256),
                   "fd23_batch_autotune")
        return [tab[k].as_dict() for k in range(min(n, 256))]


def receivers_line(nsta, ix0, iz0, idx, idz):
    """Reference line receivers: station i at (ix0+i*idx, iz0+i*idz) recorded
    as the pair (x, z), (x-1, z) (PD/record/cu_record.cu:12-28)."""
    rx = _np.zeros(2 * nsta, dtype=_np.int32)
    rz = _np.zeros(2 * nsta, dtype=_np.int32)
    _check(lib().fd23_receivers_line(nsta, ix0, iz0, idx, idz, _p(rx), _p(rz)), "receivers_line")
    return rx, rz


def receivers_file(path):
    """Station file of whitespace-separated (z x) pairs, each recorded as the
    pair (x, z), (x-1, z) (PD/record/cu_record.cu:30-76)."""
    vals = [int(t) for t in open(path).read().split()]
    rx, rz = [], []
    for j in range(0, len(vals) - 1, 2):
        z, x = vals[j], vals[j + 1]
        rx += [x, x - 1]
        rz += [z, z]
    return _np.array(rx, dtype=_np.int32), _np.array(rz, dtype=_np.int32)


def read_model(name, nx, nz, h):
    """vp, vs, den (nz, nx) FP64 from a .mdl polygon model or raster files
    <name>.vp/.vs/.den (fd23_read_model)."""
    out = [_np.empty((nz, nx)) for _ in range(3)]
    _check(lib().fd23_read_model(name.encode(), nx, nz, h, *[_p(o) for o in out]), "fd23_read_model")
    return out


def punch_tiles(nx, nz):
    """(nbx, nbz): the 32 x 16 tiles of the step windows."""
    a, b = _C.c_int(0), _C.c_int(0)
    _check(lib().fd23_punch_tiles(nx, nz, _C.byref(a), _C.byref(b)), "fd23_punch_tiles")
    return a.value, b.value


def punch_windows(times, before, after, dt, elem="f64"):
    """Tile step windows (first, last), int32 [nbz*nbx] each, from travel
    times t[nz, nx] (fd23_punch_windows; elem 'f64' as PD, 'f32' as PN/SH)."""
    es = 8 if elem == "f64" else 4
    t = _np.ascontiguousarray(times, dtype=_np.float64 if es == 8 else _np.float32)
    nz, nx = t.shape
    nbx, nbz = punch_tiles(nx, nz)
    first = _np.zeros(nbx * nbz, _np.int32)
    last = _np.zeros(nbx * nbz, _np.int32)
    _check(lib().fd23_punch_windows(_p(t), es, nx, nz, before, after, dt, _p(first), _p(last)),
           "fd23_punch_windows")
    return first, last


def read_punch(timefile, nx, nz, before, after, dt, elem="f64"):
    """The same from a raw travel-time file (the reference's `timefile`)."""
    nbx, nbz = punch_tiles(nx, nz)
    first = _np.zeros(nbx * nbz, _np.int32)
    last = _np.zeros(nbx * nbz, _np.int32)
    _check(lib().fd23_read_punch(timefile.encode(), 8 if elem == "f64" else 4, nx, nz, before, after, dt,
                                 _p(first), _p(last)), "fd23_read_punch")
    return first, last


def read_raster_model(prefix, nx, nz, wave="psv"):
    """Float32 raster model files <prefix>.vp, .vs, .den (PD/model/util.cpp:12-28)."""
    def rd(ext):
        return _np.fromfile("%s.%s" % (prefix, ext), dtype=_np.float32,
                            count=nx * nz).astype(_np.float64).reshape(nz, nx)
    vp = rd("vp") if _WAVES[wave] == PSV else None
    return vp, rd("vs"), rd("den")


# ---------------------------------------------------------------------------
class Solver:
    """One shot on one GPU (owns its device buffers)."""

    def __init__(self, wave, nx, nz, npml, h, dt, prec="f32", topabsorb=0, pml_dt=None,
                 pml_v=None, pml_r=1e-11, pml_fc=None, device=0, kernel="auto"):
        self.wave = _WAVES[wave]
        self.prec = _PRECS[prec]
        self.nx, self.nz, self.npml = nx, nz, npml
        d = Desc(self.wave, self.prec, nx, nz, npml, int(topabsorb), h, dt,
                 dt if pml_dt is None else pml_dt, 30.0 if pml_v is None else pml_v, pml_r,
                 2.0 if pml_fc is None else pml_fc, device, _KERNELS[kernel])
        self._h = _C.c_void_p()
        _check(lib().fd23_create(_C.byref(d), _C.byref(self._h)), "fd23_create")
        self.dtype = _np.float64 if self.prec == F64 else _np.float32
        self.nfields = 5 if self.wave == PSV else 3
        self._nrec = {}
        self._box = None

    def close(self):
        if self._h:
            lib().fd23_destroy(self._h)
            self._h = _C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- inputs --
    def set_model(self, vp, vs, den):
        stab = _C.c_double(0.0)
        n = self.nx * self.nz
        vp = _sized(_f64(vp), n, "vp") if vp is not None else None
        vs, den = _sized(_f64(vs), n, "vs"), _sized(_f64(den), n, "den")
        _check(lib().fd23_set_model(self._h, _p(vp), _p(vs), _p(den),
                                    _C.cast(_C.pointer(stab), _C.c_void_p)), "fd23_set_model")
        return stab.value

    def set_material(self, mat):
        nm = 5 if self.wave == PSV else 3
        _check(lib().fd23_set_material(self._h, _p(_sized(_f64(mat), nm * self.nx * self.nz, "mat"))),
               "fd23_set_material")

    def set_cpml(self, bck):
        per = 4 if self.wave == PSV else 2
        n = 3 * per * (self.nx + self.nz)
        _check(lib().fd23_set_cpml(self._h, _p(_sized(_f64(bck), n, "bck"))), "fd23_set_cpml")

    def set_source(self, kind, xs, zs, moment, src, nt_max):
        src = _f64(src)
        _check(lib().fd23_set_source(self._h, kind, xs, zs,
                                     _p(_f64(moment)) if moment is not None else None, _p(src),
                                     len(src), nt_max), "fd23_set_source")

    def set_source_terms(self, field, ix, iz, amp):
        amp = _f64(amp)
        n = len(field)
        if len(ix) != n or len(iz) != n or (n and (amp.ndim != 2 or amp.shape[0] != n)):
            raise ValueError("set_source_terms: field, ix, iz and amp rows must agree")
        _check(lib().fd23_set_source_terms(self._h, n, _p(_i32(field)), _p(_i32(ix)),
                                           _p(_i32(iz)), _p(amp), amp.shape[1] if n else 0),
               "fd23_set_source_terms")

    def set_receivers(self, field, rx, rz):
        rx, rz = _i32(rx), _i32(rz)
        if rx.size != rz.size:
            raise ValueError("set_receivers: rx and rz differ in length")
        _check(lib().fd23_set_receivers(self._h, field, _p(rx), _p(rz), len(rx)),
               "fd23_set_receivers")
        self._nrec[field] = len(rx)

    # -- time stepping --
    def run(self, nsteps, itrecord=1):
        _check(lib().fd23_run(self._h, nsteps, itrecord), "fd23_run")

    def sync(self):
        _check(lib().fd23_sync(self._h), "fd23_sync")

    @property
    def stream(self):
        """cudaStream_t (as an int) all launches of this solver use."""
        p = _C.c_void_p()
        _check(lib().fd23_get_stream(self._h, _C.byref(p)), "fd23_get_stream")
        return p.value or 0

    def field_ptrs(self):
        """Device addresses of the stored wavefields the solver currently
        reads (padded layout, storage type), valid until the next run."""
        out = []
        for f in range(5 if self.wave == PSV else 3):
            p, n = _C.c_void_p(), _C.c_size_t(0)
            _check(lib().fd23_get_field_device(self._h, f, _C.byref(p), _C.byref(n)), "fd23_get_field_device")
            out.append(p.value or 0)
        return out

    def stored_elems(self):
        """Stored elements of one wavefield (nx*nz cells plus zero padding)."""
        p, n = _C.c_void_p(), _C.c_size_t(0)
        _check(lib().fd23_get_field_device(self._h, 0, _C.byref(p), _C.byref(n)), "fd23_get_field_device")
        return n.value

    @property
    def step(self):
        it = _C.c_int(0)
        _check(lib().fd23_get_step(self._h, _C.byref(it)), "fd23_get_step")
        return it.value

    def seismograms(self, field, out=None):
        """[record rows, traces] of one field.  out: a caller-owned C-contiguous
        array of that shape and the compute type (e.g. pinned host memory) to
        copy into instead of a new array."""
        n = self._nrec.get(field, 0)
        nr = _C.c_int(0)
        _check(lib().fd23_get_seismograms(self._h, field, None, 0, _C.byref(nr)), "seismograms")
        if out is None:
            out = _np.zeros((nr.value, n), dtype=self.dtype)
        elif (out.shape != (nr.value, n) or out.dtype != _np.dtype(self.dtype) or
              not out.flags["C_CONTIGUOUS"]):
            raise ValueError("seismograms: out must be C-contiguous %s of shape %s"
                             % (_np.dtype(self.dtype).name, (nr.value, n)))
        _check(lib().fd23_get_seismograms(self._h, field, _p(out), out.nbytes, _C.byref(nr)),
               "seismograms")
        return out

    def reset(self):
        _check(lib().fd23_reset(self._h), "fd23_reset")

    def state_size(self):
        return lib().fd23_state_bytes(self._h) // _np.dtype(self.dtype).itemsize

    def get_state(self):
        out = _np.zeros(self.state_size(), dtype=self.dtype)
        _check(lib().fd23_get_state(self._h, _p(out), out.nbytes), "fd23_get_state")
        return out

    def set_state(self, state, it0):
        st = _np.ascontiguousarray(state, dtype=self.dtype)
        _check(lib().fd23_set_state(self._h, _p(st), st.nbytes, it0), "fd23_set_state")

    # -- work plan --
    def autotune(self, trial_steps=10):
        """Time the candidate work plans on this shot and keep the fastest;
        returns the trials as dicts."""
        tab = (TuneEntry * 256)()
        n = _check(lib().fd23_autotune(self._h, trial_steps, _C.cast(tab, _C.c_void_p), 256), "fd23_autotune")
        return [tab[k].as_dict() for k in range(min(n, 256))]

    def set_plan(self, wx=4.0, wz=3.0, per_sm=3, oversub=1.0, bands=1, fast_iter=0):
        """Install a work plan without timing it (fd23_set_plan); fast_iter=1
        selects the FP32 sweep with uniform fast iterations."""
        t = TuneEntry(wx=wx, wz=wz, per_sm=per_sm, bands=bands, oversub=oversub, fast_iter=fast_iter)
        _check(lib().fd23_set_plan(self._h, _C.cast(_C.pointer(t), _C.c_void_p)), "fd23_set_plan")

    def plan(self):
        """The current work plan and its CTA count (fd23_get_plan)."""
        e = TuneEntry()
        nb = _C.c_int(0)
        _check(lib().fd23_get_plan(self._h, _C.cast(_C.pointer(e), _C.c_void_p), _C.byref(nb)), "fd23_get_plan")
        d = e.as_dict()
        d["nblocks"] = nb.value
        return d

    # -- material table --
    def set_material_table(self, on=True):
        """Index + table form of the material (mktable): returns the number of
        table entries; raises Fd23Error (ERR_UNSUPPORTED) with more than 255
        distinct material tuples."""
        return _check(lib().fd23_set_material_table(self._h, 1 if on else 0), "fd23_set_material_table")

    # -- usepunch --
    def set_punch(self, first, last):
        """Tile step windows (first, last) of punch_windows / read_punch;
        None, None removes them."""
        if first is None and last is None:
            _check(lib().fd23_set_punch(self._h, None, None, 0, 0), "fd23_set_punch")
            return
        nbx, nbz = punch_tiles(self.nx, self.nz)
        f = _np.ascontiguousarray(first, dtype=_np.int32).ravel()
        l = _np.ascontiguousarray(last, dtype=_np.int32).ravel()
        if f.size != nbx * nbz or l.size != nbx * nbz:
            nbx = nbz = -1  # let the library reject the sizes
        _check(lib().fd23_set_punch(self._h, _p(f), _p(l), nbx, nbz), "fd23_set_punch")

    def set_punch_phase(self, steps):
        """Steps per phase plan of the windowed sweep (0: one static plan)."""
        _check(lib().fd23_set_punch_phase(self._h, steps), "fd23_set_punch_phase")

    # -- hybrid box --
    def set_box(self, x0, z0, bx, bz, bmat=None):
        """Box [x0, x0+bx) x [z0, z0+bz); bmat (5, bz, bx) dt/h-scaled or None
        for the cut of the grid material.  bx = bz = 0 removes it."""
        if bmat is not None:
            bmat = _sized(_f64(bmat), 5 * max(bx, 0) * max(bz, 0), "bmat")
        _check(lib().fd23_set_box(self._h, x0, z0, bx, bz, _p(bmat)), "fd23_set_box")
        self._box = (x0, z0, bx, bz) if bx else None

    def set_model_box(self, vp, vs, den, x0, z0, bx, bz, src_vp, src_vs, src_den):
        """fd23_set_model_box: the material built on the device, the box at
        (x0, z0) homogenised towards the source material and its box material
        installed (box_material + set_material + set_box(bmat) on the host);
        returns the number of box cells that took the source material and the
        FP64 box material (5, bz, bx)."""
        n = self.nx * self.nz
        vp, vs, den = (_sized(_f64(a), n, nm) for a, nm in ((vp, "vp"), (vs, "vs"), (den, "den")))
        stab = _C.c_double(0.0)
        rep = _C.c_int(0)
        bmat = _np.zeros((5, bz, bx))
        _check(lib().fd23_set_model_box(self._h, _p(vp), _p(vs), _p(den), x0, z0, bx, bz, float(src_vp),
                                        float(src_vs), float(src_den), _C.byref(stab), _C.byref(rep), _p(bmat)),
               "fd23_set_model_box")
        self._box = (x0, z0, bx, bz)
        return rep.value, bmat

    def set_box_incident(self, inc, it0=0, wait=True):
        """inc [nsteps, 5, nring] (U W Txx Txz Tzz on the ring cells) for steps
        it0 .. it0+nsteps-1.  wait=False: fd23_set_box_incident_async (the
        upload overlaps the run; the solver keeps a reference to the array
        until the next upload)."""
        a = _np.ascontiguousarray(inc, dtype=self.dtype)
        if self._box is not None:
            nring = sum(box_ring_size(self._box[2], self._box[3]))
            if a.ndim != 3 or a.shape[1:] != (5, nring):
                raise ValueError("set_box_incident: shape %s, expected (nsteps, 5, %d)" % (a.shape, nring))
        n = a.shape[0] if a.ndim == 3 else 0
        if wait:
            _check(lib().fd23_set_box_incident(self._h, _p(a), it0, n), "fd23_set_box_incident")
            self._inc_keep = None
        else:
            _check(lib().fd23_set_box_incident_async(self._h, _p(a), it0, n), "fd23_set_box_incident_async")
            self._inc_keep = a

    def set_box_line_source(self, desc, src, bmat, it0, nsteps):
        """Incident field of steps it0 .. it0+nsteps-1 generated on the device
        from the line source desc (planes (bx+8) x (bz+8)); bmat (5, bz, bx)
        FP64 box material."""
        src = _f64(src)
        if self._box is not None:
            bmat = _sized(_f64(bmat), 5 * self._box[2] * self._box[3], "bmat")
        else:
            bmat = _f64(bmat)
        _check(lib().fd23_set_box_line_source(self._h, _C.byref(desc), _p(src), len(src), _p(bmat), it0, nsteps),
               "fd23_set_box_line_source")

    def get_box_state(self):
        n = lib().fd23_box_state_bytes(self._h) // _np.dtype(self.dtype).itemsize
        out = _np.zeros(n, dtype=self.dtype)
        _check(lib().fd23_get_box_state(self._h, _p(out), out.nbytes), "fd23_get_box_state")
        return out

    def set_box_state(self, r):
        a = _np.ascontiguousarray(r, dtype=self.dtype)
        _check(lib().fd23_set_box_state(self._h, _p(a), a.nbytes), "fd23_set_box_state")

    def norm2(self):
        v = _C.c_double(0.0)
        _check(lib().fd23_field_norm2(self._h, _C.byref(v)), "fd23_field_norm2")
        return v.value
