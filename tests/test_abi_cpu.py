"""CPU checks of the C ABI library (no GPU needed): it loads, exports every
function include/fd23.h declares, and its FP64 host set-up (material, CPML,
wavelets, moment tensors, source terms, receiver lists) is bit-identical to
the oracle's restatement of the reference."""
import os
import re

import numpy as np
import pytest

import fd23_gb300 as F
from oracle import fd23_oracle as O
from tests.fd23_cases import layered_model

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "fd23.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fd23_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_function():
    lib = F.lib()
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(F.ABI_FUNCTIONS) == names


def test_tune_entry_layout(tmp_path):
    """fd23_tune_entry: bands fills the padding after per_sm, fast_iter comes
    last (48 bytes with its padding); the ctypes mirror matches the header as
    a C compiler lays it out."""
    import ctypes
    import shutil
    import subprocess
    assert ctypes.sizeof(F.TuneEntry) == 48
    assert F.TuneEntry.per_sm.offset == 16 and F.TuneEntry.bands.offset == 20
    assert F.TuneEntry.oversub.offset == 24 and F.TuneEntry.ms_per_step.offset == 32
    assert F.TuneEntry.fast_iter.offset == 40
    t = F.TuneEntry()
    assert t.bands == 0 and t.fast_iter == 0  # zero-filled: strip-major cut, plain sweep
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "fd23.h"\n'
                   'int main(void) { printf("%zu %zu %zu %zu %zu\\n", sizeof(fd23_tune_entry), '
                   'offsetof(fd23_tune_entry, bands), offsetof(fd23_tune_entry, oversub), '
                   'offsetof(fd23_tune_entry, ms_per_step), offsetof(fd23_tune_entry, fast_iter)); return 0; }\n')
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert [int(v) for v in got] == [48, 20, 24, 32, 40]


def test_create_without_gpu_fails_cleanly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(F.Fd23Error) as e:
        F.Solver("psv", 64, 64, 8, 0.3, 0.01)
    assert e.value.status == -2


def test_argument_validation():
    with pytest.raises(F.Fd23Error):
        F.Solver("psv", 64, 64, 40, 0.3, 0.01)  # 2*npml > nx
    assert F.lib().fd23_strerror(-3).decode().startswith("model fails")


@pytest.mark.parametrize("seed,fluid", [(0, False), (1, True), (2, True)])
def test_psv_material_matches_oracle(seed, fluid):
    nx, nz = 77, 53
    vp, vs, den = layered_model(nx, nz, seed, fluid_rows=(10, 16) if fluid else None)
    if fluid:
        vs[:, :3] = 0.0   # fluid cells at the left edge exercise the water-edge rule
        vs[-4:, :] = 0.0
    m, stab, rc = F.build_material("psv", vp, vs, den, 0.3, 0.01)
    mo, stabo, rco = O.psv_material(vp, vs, den, 0.3, 0.01)
    np.testing.assert_array_equal(m, mo)
    assert stab == stabo and rc == 0 == rco


def test_psv_material_golden_model(tmp_path):
    d = np.load(os.path.join(ROOT, "tests", "golden", "psv_fp64_golden.npz"))
    mdl = tmp_path / "m.mdl"
    mdl.write_text(str(d["mdl"]))
    vp, vs, den = O.mdl_raster(O.parse_mdl(str(mdl)), 300, 900, 0.3)
    m, _, _ = F.build_material("psv", vp, vs, den, 0.3, 0.01)
    mo, _, _ = O.psv_material(vp, vs, den, 0.3, 0.01)
    np.testing.assert_array_equal(m, mo)


def test_unstable_model_reported():
    vp = np.full((20, 20), 60.0)
    m, stab, rc = F.build_material("psv", vp, vp / 2, vp * 0 + 2.0, 0.3, 0.01)
    assert rc == -3 and stab > 1.0


def test_sh_material_matches_oracle():
    vp, vs, den = layered_model(61, 45, 4)
    m, stab, rc = F.build_material("sh", None, vs, den, 0.3, 0.01)
    mo, stabo, rco = O.sh_material(vs, den, 0.3, 0.01)
    np.testing.assert_array_equal(m, mo)


@pytest.mark.parametrize("wave", ["psv", "sh"])
@pytest.mark.parametrize("npml,nx,nz", [(32, 96, 96), (20, 257, 131), (7, 40, 30)])
def test_cpml_matches_oracle(wave, npml, nx, nz):
    a = F.build_cpml(wave, nx, nz, npml, 0.005, 1e-11, 30.0, 2.0)
    b = (O.cpml_psv if wave == "psv" else O.cpml_sh)(nx, nz, npml, 0.005, 1e-11, 30.0, 2.0)
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("alpha", [-30, -20, -5, 0, 4])
def test_gaussian_matches_oracle(alpha):
    np.testing.assert_array_equal(F.wavelet_gaussian(0.01, alpha), O.gaussian(0.01, alpha))


def test_trapezoid_and_ricker():
    np.testing.assert_array_equal(F.wavelet_trapezoid(0.01, 0.3, 0.0, 0.3),
                                  O.trapezoid(0.01, 0.3, 0.0, 0.3))
    np.testing.assert_allclose(F.wavelet_ricker(4e-4, 15.0), O.ricker(4e-4, 15.0), rtol=0,
                               atol=1e-18)


@pytest.mark.parametrize("angles", [(0, 90, 0, 45), (0, 20, 90, 45), (30, 60, -45, 10)])
def test_moments_match_oracle(angles):
    np.testing.assert_array_equal(F.moment_psv(*angles), O.moment_psv(*angles))
    np.testing.assert_array_equal(F.moment_sh(*angles), O.moment_sh(*angles))


@pytest.mark.parametrize("wave,kinds", [("psv", (1, 3, 13)), ("sh", (2, 3, 13))])
def test_source_terms_match_oracle(wave, kinds):
    src = O.gaussian(0.01, -5)
    m = O.moment_psv(0, 20, 90, 45) if wave == "psv" else O.moment_sh(0, 20, 90, 45)
    for kind in kinds:
        f, x, z, amp = F.build_source_terms(wave, kind, 40, 30, m, 0.3, 0.01, src, 80)
        fo, io, ao = O.source_terms(wave, kind, 100, 40, 30, m, 0.3, 0.01, src, 80)
        np.testing.assert_array_equal(f, fo)
        np.testing.assert_array_equal(x + z * 100, io)
        np.testing.assert_array_equal(amp, ao)


def test_receiver_lists():
    rx, rz = F.receivers_line(5, 513, 0, 2, 0)
    orx, orz = O.receivers_line(5, 513, 0, 2, 0)
    np.testing.assert_array_equal(rx, orx)
    np.testing.assert_array_equal(rz, orz)
