"""fd23_psv2d on the GPU: the program's trace files equal the same run through
the API bit for bit (FP32 and FP64), its .isis files carry the reference's
header layout, and savestate / restart split a run exactly."""
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
    vp, vs, den = F.read_model(str(tmp_path / "layers.mdl"), 150, 100, np.float32(0.3))
    s = F.Solver("psv", 150, 100, 12, float(np.float32(0.3)), float(np.float32(0.01)), prec=prec, pml_dt=0.005,
                 pml_v=30.0, pml_r=1e-11, pml_fc=2.0)
    s.set_model(vp, vs, den)
    src = F.wavelet_gaussian(float(np.float32(0.01)), -5)
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
