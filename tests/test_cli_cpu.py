"""Model / station input and the parfile program, CPU side: the product's
.mdl reader against the oracle's restatement (the FP64 golden's model and a
model with named vertices and overlapping polygons), raster and station
files, and fd23_psv2d's parameter handling (dry runs, no GPU)."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import fd23_oracle as O

F = pytest.importorskip("fd23_gb300")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "fd23_gb300", "_lib", "fd23_psv2d")
CLI_SH = os.path.join(ROOT, "fd23_gb300", "_lib", "fd23_sh2d")

MDL_DEFS = """# overlapping polygons, named vertices, negative vs / den as factors of vp
DEF a 10 5
DEF b 50 5
DEF c 50 30
DEF d 10 30
BACK 5.0 -0.577 -0.62
POLY 6.0 3.4 2.7
\ta b c d
POLY 7.0 4.0 3.0
\t30 0 70 0
\t70 20 30 20
"""


def _lib_or_skip():
    try:
        F.lib()
    except ImportError as e:
        pytest.skip(str(e))


@pytest.mark.parametrize("which", ["golden", "defs"])
def test_read_model_matches_oracle(tmp_path, which):
    _lib_or_skip()
    if which == "golden":
        g = np.load(os.path.join(ROOT, "tests", "golden", "psv_fp64_golden.npz"))
        text = str(g["mdl"])
        nx, nz, h = 2048, 1024, 0.3
    else:
        text, nx, nz, h = MDL_DEFS, 97, 43, 0.7
    path = tmp_path / "m.mdl"
    path.write_text(text)
    got = F.read_model(str(path), nx, nz, h)
    want = O.mdl_raster(O.parse_mdl(str(path)), nx, nz, h)
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)
    if which == "defs":
        assert len(np.unique(got[0])) == 3  # background and both polygons present


def test_read_raster_model_and_stations(tmp_path):
    _lib_or_skip()
    nx, nz = 31, 17
    rng = np.random.default_rng(3)
    arrs = [rng.uniform(1, 5, (nz, nx)).astype(np.float32) for _ in range(3)]
    for a, ext in zip(arrs, ("vp", "vs", "den")):
        a.tofile(str(tmp_path / ("m." + ext)))
    got = F.read_model(str(tmp_path / "m"), nx, nz, 1.0)
    for a, b in zip(got, arrs):
        np.testing.assert_array_equal(a, b.astype(np.float64))
    with pytest.raises(F.Fd23Error):
        F.read_model(str(tmp_path / "missing"), nx, nz, 1.0)
    st = tmp_path / "stations"
    st.write_text("0 10\n3 20\n 5 7\n")
    import ctypes
    n = F.lib().fd23_read_stations(str(st).encode(), None, None, 0)
    assert n == 6
    rx = np.zeros(n, np.int32)
    rz = np.zeros(n, np.int32)
    F.lib().fd23_read_stations(str(st).encode(), rx.ctypes.data_as(ctypes.c_void_p),
                                rz.ctypes.data_as(ctypes.c_void_p), n)
    wx, wz = O.receivers_file(str(st))
    np.testing.assert_array_equal(rx, wx)
    np.testing.assert_array_equal(rz, wz)


PAR = """# reference-style parameter file
nx=120 nz=90 nt=40 h=0.3 dt=0.01
srctime=Gaussian alpha=-5
strike=0 dip=20 rake=90 azimuth=45
xs=60 zs=30
npml=12 pml_dt=0.005 pml_v=30 pml_fc=2 pml_r=1e-11
output=out model=m.mdl ntsnap=100 gpuid=1
nrec=10 ixrec0=5 izrec0_u=0 izrec0_w=1 idxrec=9 idzrec=0
"""


def _cli(tmp_path, *args):
    if not os.path.exists(CLI):
        pytest.skip("fd23_psv2d not built")
    return subprocess.run([CLI] + list(args), cwd=str(tmp_path), capture_output=True, text=True)


def test_cli_parameters(tmp_path):
    (tmp_path / "run.par").write_text(PAR)
    r = _cli(tmp_path, "par=run.par", "dryrun=1")
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    assert (d["nx"], d["nz"], d["nt"], d["npml"], d["traces_u"], d["source"]) == (120, 90, 40, 12, 20, "moment")
    assert d["lsrc"] == len(O.gaussian(0.01, -5))
    # later words win, on the command line and across files
    r = _cli(tmp_path, "nt=7", "par=run.par", "nt=9", "srctype=p", "prec=f64", "explosion=1", "dryrun=1")
    d = json.loads(r.stdout)
    assert (d["nt"], d["prec"], d["source"]) == (9, "f64", "explosion")
    # station files replace the receiver line
    (tmp_path / "st").write_text("0 10\n0 20\n0 30\n")
    d = json.loads(_cli(tmp_path, "par=run.par", "U_sta_file=st", "W_sta_file=st", "dryrun=1").stdout)
    assert d["traces_u"] == d["traces_w"] == 6
    # trapezoid source time function
    d = json.loads(_cli(tmp_path, "par=run.par", "srctime=Trapezoid", "trap1=0.1", "trap2=0.05", "trap3=0.1",
                        "dryrun=1").stdout)
    assert d["lsrc"] == len(O.trapezoid(0.01, 0.1, 0.05, 0.1))


def test_cli_errors(tmp_path):
    (tmp_path / "run.par").write_text(PAR)
    r = _cli(tmp_path, "par=run.par", "srctype=x", "dryrun=1")
    assert r.returncode == 1 and "srctype" in r.stderr
    r = _cli(tmp_path, "nx=10", "dryrun=1")
    assert r.returncode == 1 and "missing parameter" in r.stderr
    r = _cli(tmp_path, "par=nofile.par")
    assert r.returncode == 1
    r = _cli(tmp_path, "par=run.par", "usepunch=1", "dryrun=1")
    assert r.returncode == 1 and "usepunch" in r.stderr
    r = _cli(tmp_path, "par=run.par", "prec=f8", "dryrun=1")
    assert r.returncode == 1


def test_cli_usepunch_windows(tmp_path):
    """usepunch=1 reads the float travel-time file (double with prec=f64) and
    builds the windows of PN/slide/cu_slide.cu (checked against the oracle)."""
    (tmp_path / "run.par").write_text(PAR)
    rng = np.random.default_rng(9)
    t = rng.uniform(0.05, 2.0, size=(90, 120))
    t.astype(np.float32).tofile(str(tmp_path / "tt32"))
    t.tofile(str(tmp_path / "tt64"))
    for prec, name, elem in (("f32", "tt32", "f32"), ("f64", "tt64", "f64")):
        r = _cli(tmp_path, "par=run.par", "usepunch=1", "before=0.1", "after=0.3", "timefile=" + name,
                 "prec=" + prec, "dryrun=1")
        assert r.returncode == 0, r.stderr
        d = json.loads(r.stdout)
        first, _ = O.punch_windows(t.astype(np.float32) if elem == "f32" else t, 0.1, 0.3, 0.01, elem)
        assert d["punch_tiles"] == len(first) == 4 * 6
        assert d["punch_first_min"] == first.min()
    r = _cli(tmp_path, "par=run.par", "usepunch=1", "before=0.1", "after=0.3", "timefile=none", "dryrun=1")
    assert r.returncode == 1 and "timefile" in r.stderr


SH_PAR = """nx=200 nz=100 nt=20 h=10 dt=0.001
sourcetime=Gaussian alpha=-5
strike=0 dip=90 rake=0 azimuth=45
xs=100 zs=20 npml=20 pml_dt=0.001 pml_v=300 pml_fc=10 pml_r=1e-11
itrecord=1 output=sh model=m.mdl ntsnap=100 ngpu=1 usepunch=0
nrec=20 ixrec0=5 izrec0_v=0 idxrec=9 idzrec=0
"""


def test_sh_program_parameters(tmp_path):
    if not os.path.exists(CLI_SH):
        pytest.skip("fd23_sh2d not built")
    (tmp_path / "sh.par").write_text(SH_PAR)
    run = lambda *a: subprocess.run([CLI_SH, "par=sh.par"] + list(a), cwd=str(tmp_path), capture_output=True,
                                    text=True)
    d = json.loads(run("dryrun=1").stdout)
    assert (d["source"], d["traces_u"], d["nx"]) == ("moment", 40, 200)
    assert json.loads(run("stype=13", "dryrun=1").stdout)["source"] == "moment_p"
    assert json.loads(run("stype=2", "dryrun=1").stdout)["source"] == "force"
    assert run("stype=5", "dryrun=1").returncode == 1
    (tmp_path / "st").write_text("0 10\n0 30\n")
    assert json.loads(run("V_sta_file=st", "dryrun=1").stdout)["traces_u"] == 4


NTDE = os.path.join(os.path.dirname(CLI), "fd23_ntde_line")


def test_usebox_parameters(tmp_path):
    """usebox=1: the box around (xs, zs), the reference's boundary check on
    zs, and the options a box run excludes."""
    (tmp_path / "run.par").write_text(PAR)
    box = ["usebox=1", "srcden=2.6", "srcsvel=3.2", "srcpvel=5.5", "sourcefile=pl.bin", "bw=20", "zs=40", "xs=60"]
    r = _cli(tmp_path, "par=run.par", "dryrun=1", "prec=f64", *box)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    assert d["box"] == [60 + 10 + 1 - 20, 40 + 10 + 1 - 20, 20, 20] and d["boxsource"] == "pl.bin"
    d = json.loads(_cli(tmp_path, "par=run.par", "dryrun=1", *box, "boxsource=device").stdout)
    assert d["boxsource"] == "device"
    r = _cli(tmp_path, "par=run.par", "dryrun=1", *box, "zs=13")  # bw/2 + 4 = 14
    assert r.returncode == 1 and "too near" in r.stderr
    r = _cli(tmp_path, "par=run.par", "dryrun=1", *box, "usepunch=1", "before=0", "after=1", "timefile=t")
    assert r.returncode == 1 and "usebox" in r.stderr
    r = _cli(tmp_path, "par=run.par", "dryrun=1", *box, "prec=bf16")
    assert r.returncode == 1 and "usebox" in r.stderr
    r = _cli(tmp_path, "par=run.par", "dryrun=1", "usebox=1", "bw=20")
    assert r.returncode == 1 and "missing parameter" in r.stderr and "srcden" in r.stderr


def test_ntde_program_parameters(tmp_path):
    if not os.path.exists(NTDE):
        pytest.skip("fd23_ntde_line not built")
    r = subprocess.run([NTDE, "nt=10", "h=1", "dt=0.001"], cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 1 and "missing parameter" in r.stderr and "sourcefile" in r.stderr
    r = subprocess.run([NTDE, "nt=10", "h=1", "dt=0.001", "srcden=2", "srcsvel=2", "srcpvel=3", "bw=8",
                        "sourcefile=x.bin", "sourcetime=none", "strike=0", "dip=0", "rake=0", "azimuth=0"],
                       cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode == 1 and "sourcetime" in r.stderr
