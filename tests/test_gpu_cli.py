"""fd23_psv2d on the GPU: the program's trace files equal the same run through
the API bit for bit (FP32 and FP64), its .isis files carry the reference's
header layout, and savestate / restart split a run exactly; fd23_ntde_line
writes the box-source planes and fd23_psv2d usebox=1 runs the hybrid box
from them."""
import os
import struct
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "fd23_gb300", "_lib", "fd23_psv2d")
CLI_SH = os.path.join(ROOT, "fd23_gb300", "_lib", "fd23_sh2d")

MDL = """BACK 5.5 3.2 2.6
POLY 6.5 3.7 2.9
\t-10 12
\t100 9
\t100 40
\t-10 40
"""
PAR = """nx=150 nz=100 h=0.3 dt=0.01
srctime=Gaussian alpha=-5
strike=0 dip=20 rake=90 azimuth=45
xs=75 zs=20
npml=12 pml_dt=0.005 pml_v=30 pml_fc=2 pml_r=1e-11
model=layers.mdl ntsnap=100
U_sta_file=st W_sta_file=st
"""
STATIONS = [(0, 10), (0, 40), (1, 80), (0, 120), (20, 60)]


def _setup(tmp_path):
    if not os.path.exists(CLI):
        pytest.skip("fd23_psv2d not built")
    (tmp_path / "layers.mdl").write_text(MDL)
    (tmp_path / "run.par").write_text(PAR)
    (tmp_path / "st").write_text("".join("%d %d\n" % zx for zx in STATIONS))


def _cli(tmp_path, *args):
    r = subprocess.run([CLI, "par=run.par"] + list(args), cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def _api(tmp_path, prec, nt):
    # the program reads h and dt as doubles for f64 (PD), as floats otherwise (PN)
    h, dt = (0.3, 0.01) if prec == "f64" else (float(np.float32(0.3)), float(np.float32(0.01)))
    vp, vs, den = F.read_model(str(tmp_path / "layers.mdl"), 150, 100, h)
    s = F.Solver("psv", 150, 100, 12, h, dt, prec=prec, pml_dt=0.005, pml_v=30.0, pml_r=1e-11, pml_fc=2.0)
    s.set_model(vp, vs, den)
    src = F.wavelet_gaussian(dt, -5)
    s.set_source(F.SRC_MOMENT, 75, 20, F.moment_psv(0, 20, 90, 45), src, nt)
    rx, rz = F.receivers_file(str(tmp_path / "st"))
    s.set_receivers(0, rx, rz)
    s.set_receivers(1, rx, rz)
    s.run(nt, 1)
    out = s.seismograms(0), s.seismograms(1)
    s.close()
    return out


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_cli_equals_api(tmp_path, prec):
    _setup(tmp_path)
    nt = 60
    _cli(tmp_path, "nt=%d" % nt, "output=run", "prec=" + prec)
    dt = np.float64 if prec == "f64" else np.float32
    su, sw = _api(tmp_path, prec, nt)
    ntr = 2 * len(STATIONS)
    fu = np.fromfile(str(tmp_path / "run_U"), dtype=dt).reshape(nt, ntr)
    fw = np.fromfile(str(tmp_path / "run_W"), dtype=dt).reshape(nt, ntr)
    np.testing.assert_array_equal(fu, su)
    np.testing.assert_array_equal(fw, sw)
    if prec == "f64":
        # the FP64 program's trace files: 136-byte double header, double samples
        for name, seis, sx, sz in (("run_U.db.isis", su, 0.5, 0.0), ("run_W.db.isis", sw, 0.0, -0.5)):
            raw = (tmp_path / name).read_bytes()
            assert len(raw) == ntr * (136 + 8 * nt)
            for r in (0, 3, ntr - 1):
                rec = raw[r * (136 + 8 * nt):(r + 1) * (136 + 8 * nt)]
                z, x = STATIONS[r // 2]
                x = x - (r % 2)
                xs, _, zs, xr, _, zr = struct.unpack("<6d", rec[:48])
                assert xr == (x + sx) * 0.3 and zr == (z + sz) * 0.3
                assert xs == (75 + 0.25) * 0.3 and zs == (20 - 0.25) * 0.3
                np.testing.assert_array_equal(np.frombuffer(rec[136:], dtype=np.float64), seis[:, r])
        return
    # .isis: per receiver an 84-byte header and nt float samples
    for name, seis, sx, sz in (("run_U.isis", su, 0.5, 0.0), ("run_W.isis", sw, 0.0, -0.5)):
        raw = (tmp_path / name).read_bytes()
        assert len(raw) == ntr * (84 + 4 * nt)
        h = np.float32(0.3)
        for r in (0, 3, ntr - 1):
            rec = raw[r * (84 + 4 * nt):(r + 1) * (84 + 4 * nt)]
            hdr = struct.unpack("<7fif3i3f4H4i", rec[:84])
            z, x = STATIONS[r // 2]
            x = x - (r % 2)
            assert hdr[3] == np.float32(np.float32(x + np.float32(sx)) * h)     # xr
            assert hdr[5] == np.float32(np.float32(z + np.float32(sz)) * h)     # zr
            assert hdr[0] == np.float32(75 * h) and hdr[2] == np.float32(20 * h)  # xs, zs
            assert hdr[7] == nt and hdr[8] == np.float32(0.01)                  # nt, samplerate
            assert hdr[9] == 75 and hdr[10] == x                                 # source / receiver flag numbers
            assert hdr[20] == 123456789 and hdr[21] == 123456789
            np.testing.assert_array_equal(np.frombuffer(rec[84:], dtype=np.float32),
                                          seis[:, r].astype(np.float32))


def test_cli_restart(tmp_path):
    _setup(tmp_path)
    _cli(tmp_path, "nt=60", "output=full")
    _cli(tmp_path, "nt=30", "output=first", "savestate=1")
    assert (tmp_path / "state000029").exists()
    _cli(tmp_path, "nt=30", "output=second", "restart=1", "nt0=30")
    ntr = 2 * len(STATIONS)
    full = np.fromfile(str(tmp_path / "full_U"), dtype=np.float32).reshape(60, ntr)
    first = np.fromfile(str(tmp_path / "first_U"), dtype=np.float32).reshape(30, ntr)
    second = np.fromfile(str(tmp_path / "second_U"), dtype=np.float32).reshape(30, ntr)
    np.testing.assert_array_equal(first, full[:30])
    np.testing.assert_array_equal(second, full[30:])


def test_cli_usepunch_equals_api(tmp_path):
    """usepunch=1 in the program = the API run with the same windows."""
    _setup(tmp_path)
    nt = 60
    zz, xx = np.mgrid[0:100, 0:150]
    t = (np.hypot(xx - 75, zz - 20) * 0.3 / 65.0).astype(np.float32)  # windows close within the run
    t.tofile(str(tmp_path / "tt"))
    _cli(tmp_path, "nt=%d" % nt, "output=pun", "usepunch=1", "before=0.05", "after=0.2", "timefile=tt")
    first, last = F.read_punch(str(tmp_path / "tt"), 150, 100, 0.05, 0.2, float(np.float32(0.01)), "f32")
    assert last.min() < nt  # some tiles close again within the run
    vp, vs, den = F.read_model(str(tmp_path / "layers.mdl"), 150, 100, np.float32(0.3))
    s = F.Solver("psv", 150, 100, 12, float(np.float32(0.3)), float(np.float32(0.01)), prec="f32", pml_dt=0.005,
                 pml_v=30.0, pml_r=1e-11, pml_fc=2.0)
    s.set_model(vp, vs, den)
    s.set_source(F.SRC_MOMENT, 75, 20, F.moment_psv(0, 20, 90, 45), F.wavelet_gaussian(float(np.float32(0.01)), -5),
                 nt)
    rx, rz = F.receivers_file(str(tmp_path / "st"))
    s.set_receivers(0, rx, rz)
    s.set_punch(first, last)
    s.run(nt, 1)
    want = s.seismograms(0)
    s.close()
    got = np.fromfile(str(tmp_path / "pun_U"), dtype=np.float32).reshape(nt, len(rx))
    np.testing.assert_array_equal(got, want)


def test_cli_usetable_equals_plain(tmp_path):
    """usetable=1 (the polygon model fits a table) writes the same traces."""
    _setup(tmp_path)
    _cli(tmp_path, "nt=40", "output=plain")
    r = _cli(tmp_path, "nt=40", "output=tab", "usetable=1")
    assert "material table:" in r.stdout
    a = np.fromfile(str(tmp_path / "plain_U"), dtype=np.float32)
    b = np.fromfile(str(tmp_path / "tab_U"), dtype=np.float32)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("stype", [3, 2])
def test_sh_program_equals_api(tmp_path, stype):
    _setup(tmp_path)
    if not os.path.exists(CLI_SH):
        pytest.skip("fd23_sh2d not built")
    nt = 50
    par = PAR.replace("srctime=", "sourcetime=").replace("U_sta_file=st W_sta_file=st", "V_sta_file=st")
    (tmp_path / "sh.par").write_text(par)
    r = subprocess.run([CLI_SH, "par=sh.par", "nt=%d" % nt, "output=shr", "stype=%d" % stype], cwd=str(tmp_path),
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    vp, vs, den = F.read_model(str(tmp_path / "layers.mdl"), 150, 100, np.float32(0.3))
    s = F.Solver("sh", 150, 100, 12, float(np.float32(0.3)), float(np.float32(0.01)), prec="f32", pml_dt=0.005,
                 pml_v=30.0, pml_r=1e-11, pml_fc=2.0)
    s.set_model(None, vs, den)
    kind = F.SRC_FORCE if stype == 2 else F.SRC_MOMENT
    s.set_source(kind, 75, 20, F.moment_sh(0, 20, 90, 45), F.wavelet_gaussian(float(np.float32(0.01)), -5), nt)
    rx, rz = F.receivers_file(str(tmp_path / "st"))
    s.set_receivers(0, rx, rz)
    s.run(nt, 1)
    want = s.seismograms(0)
    s.close()
    got = np.fromfile(str(tmp_path / "shr_V"), dtype=np.float32).reshape(nt, len(rx))
    np.testing.assert_array_equal(got, want)
    assert (tmp_path / "shr_V.isis").stat().st_size == len(rx) * (84 + 4 * nt)


CLI_NTDE = os.path.join(ROOT, "fd23_gb300", "_lib", "fd23_ntde_line")
BOX_PAR = """nx=150 nz=100 nt=60 h=0.3 dt=0.01
sourcetime=Gaussian alpha=-5
strike=30 dip=60 rake=90 azimuth=45
xs=110 zs=70
npml=12 pml_dt=0.005 pml_v=30 pml_fc=2 pml_r=1e-11
model=layers.mdl ntsnap=100
U_sta_file=stb W_sta_file=stb
usebox=1 usepunch=0 ngpu=1 srcden=2.6 srcsvel=3.2 srcpvel=5.5 sourcefile=planes.bin bw=32
"""
BOX_STATIONS = [(50, 100), (60, 90), (75, 131), (91, 110), (70, 112), (0, 110)]  # (z, x) near and in the box


def _box_api(tmp_path, prec, nt, inc=None, line=None):
    """The box run of BOX_PAR through the API (h, dt as the program reads them)."""
    h, dt = (0.3, 0.01) if prec == "f64" else (float(np.float32(0.3)), float(np.float32(0.01)))
    vp, vs, den = F.read_model(str(tmp_path / "layers.mdl"), 150, 100, h)
    mat, stab, rc = F.build_material("psv", vp, vs, den, h, dt)
    assert rc == 0
    bw, x0, z0 = 32, 110 + 16 + 1 - 32, 70 + 16 + 1 - 32
    mat, bmat, _ = F.box_material(mat, x0, z0, bw, bw, 5.5, 3.2, 2.6, dt, h)
    s = F.Solver("psv", 150, 100, 12, h, dt, prec=prec, pml_dt=0.005, pml_v=30.0, pml_r=1e-11, pml_fc=2.0)
    s.set_material(mat)
    rx, rz = F.receivers_file(str(tmp_path / "stb"))
    s.set_receivers(0, rx, rz)
    s.set_receivers(1, rx, rz)
    s.set_box(x0, z0, bw, bw, bmat=bmat)
    if inc is not None:
        s.set_box_incident(inc(bmat, dt).astype(s.dtype), 0)
    else:
        d = F.line_desc(bw + 8, bw + 8, F.line_plane_origin(bw), F.line_plane_origin(bw), h, dt, 5.5, 3.2, 2.6,
                        F.line_source_coefs(30, 60, 90, 45))
        s.set_box_line_source(d, F.wavelet_gaussian(dt, -5), bmat, 0, nt)
    s.run(nt, 1)
    out = s.seismograms(0), s.seismograms(1), mat, bmat
    s.close()
    return out


def _file_incident(planes, nt):
    """BOX::setboxsource over the file's frames: step it reads frame it + 1;
    past the end of the file the buffer keeps frame it - 1 (the reference's
    failed read leaves it)."""
    def inc(bmat, dt):
        out = []
        for it in range(nt):
            new = planes[it + 1] if it + 1 < len(planes) else planes[it - 1]
            out.append(F.box_incident_from_displacement(32, 32, dt, bmat, planes[it, 0], planes[it, 1], new[0],
                                                        new[1]))
        return np.stack(out)
    return inc


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_ntde_and_usebox_programs(tmp_path, prec):
    """fd23_ntde_line writes the generator's planes (= the API's, bit for
    bit); fd23_psv2d usebox=1 reading them equals the API box run with the
    same incident field (the reference's read order), and for FP64 the
    oracle's box run; boxsource=device equals it up to the last step, whose
    frame lies past the file's end."""
    _setup(tmp_path)
    if not os.path.exists(CLI_NTDE):
        pytest.skip("fd23_ntde_line not built")
    (tmp_path / "run.par").write_text(BOX_PAR)
    (tmp_path / "stb").write_text("".join("%d %d\n" % zx for zx in BOX_STATIONS))
    nt = 60
    r = subprocess.run([CLI_NTDE, "par=run.par"], cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    planes = np.fromfile(str(tmp_path / "planes.bin"), dtype=np.float64).reshape(nt, 2, 40, 40)
    d = F.line_desc(40, 40, F.line_plane_origin(32), F.line_plane_origin(32), 0.3, 0.01, 5.5, 3.2, 2.6,
                    F.line_source_coefs(30, 60, 90, 45))
    np.testing.assert_array_equal(planes, F.line_source_planes(d, F.wavelet_gaussian(0.01, -5), 0, nt))
    _cli(tmp_path, "output=box", "prec=" + prec)
    ntr = 2 * len(BOX_STATIONS)
    dt_ = np.float64 if prec == "f64" else np.float32
    fu = np.fromfile(str(tmp_path / "box_U"), dtype=dt_).reshape(nt, ntr)
    fw = np.fromfile(str(tmp_path / "box_W"), dtype=dt_).reshape(nt, ntr)
    su, sw, mat, bmat = _box_api(tmp_path, prec, nt, inc=_file_incident(planes, nt))
    np.testing.assert_array_equal(fu, su)
    np.testing.assert_array_equal(fw, sw)
    assert np.abs(fu).max() > 0
    if prec == "f64":
        from oracle import fd23_oracle as O
        rx, rz = F.receivers_file(str(tmp_path / "stb"))
        rec = (rx + rz * 150).astype(np.int64)
        rf = np.repeat(np.arange(2, dtype=np.int32), len(rec))
        bck = O.cpml_psv(150, 100, 12, 0.005, 1e-11, 30.0, 2.0)
        no_source = (np.zeros(0, np.int32), np.zeros(0, np.int64), np.zeros((0, 1)))
        seis, _, _ = O.psv_box_run("f64", 150, 100, 12, 0, mat, bck, no_source, rf, np.tile(rec, 2), nt,
                                   (110 + 16 + 1 - 32, 70 + 16 + 1 - 32, 32, 32), bmat,
                                   _file_incident(planes, nt)(bmat, 0.01))
        np.testing.assert_array_equal(fu, seis[:, :len(rec)])
        np.testing.assert_array_equal(fw, seis[:, len(rec):])
    # the planes generated on the device: the same run but for the last step
    _cli(tmp_path, "output=dev", "prec=" + prec, "boxsource=device")
    du = np.fromfile(str(tmp_path / "dev_U"), dtype=dt_).reshape(nt, ntr)
    if prec == "f64":
        np.testing.assert_array_equal(du[:-1], fu[:-1])
    else:  # the f32 program generates with h and dt rounded to float, the file has PD's doubles
        np.testing.assert_allclose(du[:-1], fu[:-1], rtol=0, atol=1e-5 * np.abs(fu).max())
    gu, _, _, _ = _box_api(tmp_path, prec, nt, line=True)
    np.testing.assert_array_equal(du, gu)


# header bytes the reference leaves uninitialised (stack garbage in its files):
# FP64 -- padding after nt and after status, recorder/chan/scomp/rcomp,
# user[0], user[3]; FP32 -- recorder/chan/scomp/rcomp, user[0], user[3]
_DB_UNSET = [(60, 64), (84, 88), (112, 124), (132, 136)]
_F32_UNSET = [(60, 72), (80, 84)]


def _mask(n, unset):
    m = np.ones(n, dtype=bool)
    for a, b in unset:
        m[a:b] = False
    return m


def test_fp64_program_reproduces_reference_outputs(tmp_path):
    """prec=f64 on the FP64 golden's configuration (PSV/psv_clean_double/test/
    0.par: 2048 x 1024, 2001 steps, homo.mdl with its fluid layer, 18 stations):
    0_U / 0_W equal the reference's files bit for bit, and 0_U.db.isis /
    0_W.db.isis equal the reference's trace files byte for byte outside the
    header words it leaves uninitialised."""
    if not os.path.exists(CLI):
        pytest.skip("fd23_psv2d not built")
    import json
    gold = np.load(os.path.join(ROOT, "tests", "golden", "psv_fp64_golden.npz"))
    hdr = np.load(os.path.join(ROOT, "tests", "golden", "isis_headers.npz"))
    p = json.loads(str(gold["params"]))
    (tmp_path / "homo.mdl").write_text(str(gold["mdl"]))
    (tmp_path / "sta").write_text("".join("%d %d\n" % (z, x) for z, x in gold["stations_zx"]))
    par = ("nx=%(nx)d nz=%(nz)d h=%(h)r dt=%(dt)r nt=%(nt)d xs=%(xs)d zs=%(zs)d strike=%(strike)r dip=%(dip)r "
           "rake=%(rake)r azimuth=%(azimuth)r sourcetime=Gaussian alpha=%(alpha)d stype=%(stype)d "
           "npml=%(npml)d pml_r=%(pml_r)r pml_dt=%(pml_dt)r pml_v=%(pml_v)r pml_fc=%(pml_fc)r "
           "itrecord=%(itrecord)d usebox=0 bw=24 src_shift_x=0.25 src_shift_z=-0.25 model=homo.mdl "
           "U_sta_file=sta W_sta_file=sta output=0 ntsnap=1000 ord=8 ngpu=1 usepunch=0\n") % p
    (tmp_path / "0.par").write_text(par)
    r = subprocess.run([CLI, "par=0.par", "prec=f64"], cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    nt, ntr = p["nt"], 2 * len(gold["stations_zx"])
    for c, key in (("U", "seis_u"), ("W", "seis_w")):
        got = np.fromfile(str(tmp_path / ("0_" + c)), dtype=np.float64).reshape(nt, ntr)
        np.testing.assert_array_equal(got, gold[key])
        raw = np.frombuffer((tmp_path / ("0_%s.db.isis" % c)).read_bytes(), dtype=np.uint8)
        step = 136 + 8 * nt
        assert raw.size == ntr * step
        raw = raw.reshape(ntr, step)
        m = _mask(136, _DB_UNSET)
        np.testing.assert_array_equal(raw[:, :136][:, m], hdr["fp64_" + c][:, m])
        np.testing.assert_array_equal(raw[:, 136:].copy().view(np.float64), gold[key].T)


def test_fp32_trace_headers_match_reference_layout(tmp_path):
    """The FP32 program's 84-byte headers against the reference's own
    PSV/t/clean_nobox/TEST/output_U.isis (its run: xs 512, zs 4, h 0.3,
    dt 0.01, 2000 steps, a line of 200 stations from x 513 every 2 cells,
    recorded as pairs).  The wavefield of that run is not reproducible (its
    model and receivers differ from the committed parfile), but every
    header word it sets depends only on the geometry: a run with the same
    geometry on a small grid writes the same header bytes outside the
    words the reference leaves uninitialised."""
    if not os.path.exists(CLI):
        pytest.skip("fd23_psv2d not built")
    hdr = np.load(os.path.join(ROOT, "tests", "golden", "isis_headers.npz"))["fp32_U"]
    (tmp_path / "m.mdl").write_text("BACK 6.8 4.0 3.0\n")
    par = ("nx=1024 nz=40 h=0.3 dt=0.01 nt=2000 xs=512 zs=4 srctype=1 srctime=g alpha=-20 strike=0 dip=90 "
           "rake=0 azimuth=45 npml=8 pml_r=1e-11 pml_dt=0.005 pml_v=30.0 pml_fc=2 itrecord=1 output=output "
           "nrec=200 ixrec0=513 izrec0_u=0 izrec0_w=1 idxrec=2 idzrec=0 model=m.mdl\n")
    (tmp_path / "p.par").write_text(par)
    r = subprocess.run([CLI, "par=p.par"], cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.frombuffer((tmp_path / "output_U.isis").read_bytes(), dtype=np.uint8)
    step = 84 + 4 * 2000
    assert raw.size == 400 * step
    m = _mask(84, _F32_UNSET)
    np.testing.assert_array_equal(raw.reshape(400, step)[:, :84][:, m], hdr[:, m])
