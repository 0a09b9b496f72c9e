"""The 16-bit storage forms build their material on the device: the FP64
material of the host builders, the power-of-two scale kappa from the two
material groups' maxima, and the host conversion's rounding.  A shot set up
from vp, vs, density (fd23_set_model) equals, bit for bit, the same shot set
up from the host-built FP64 material (fd23_set_material), for P-SV and SH,
BF16 and FP16, including a second model that reuses kappa."""
import numpy as np
import pytest

from oracle import fd23_oracle as O
from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu

F = pytest.importorskip("fd23_gb300")


def _shot(c, prec, mat=None, second=None):
    s = F.Solver(c.wave, c.nx, c.nz, c.npml, c.h, c.dt, prec=prec, topabsorb=c.topabsorb, **c.pml)
    if mat is None:
        s.set_model(c.vp if c.wave == "psv" else None, c.vs, c.den)
    else:
        s.set_material(mat)
    s.set_source(c.kind, c.xs, c.zs, c.m, c.src, c.nt)
    s.set_receivers(0, c.rx, c.rz)
    s.run(c.nt, 1)
    out = [s.seismograms(0), s.get_state()]
    if second is not None:  # a new model on the same solver: kappa stays
        vp2, vs2, den2, mat2 = second
        if mat is None:
            s.set_model(vp2 if c.wave == "psv" else None, vs2, den2)
        else:
            s.set_material(mat2)
        s.reset()
        s.run(c.nt, 1)
        out += [s.get_state()]
    s.close()
    return out


@pytest.mark.parametrize("prec", ["bf16", "f16"])
@pytest.mark.parametrize("wave", ["psv", "sh"])
def test_device_material_equals_host_material(wave, prec):
    c = Case(wave, 230, 150, npml=12, nt=60, seed=13, topabsorb=1, fluid=wave == "psv", zs=8)
    vp2, vs2, den2 = c.vp * 1.1, c.vs * 0.95, c.den * 1.02
    if wave == "psv":
        mat2, _, rc = O.psv_material(vp2, vs2, den2, c.h, c.dt)
    else:
        mat2, _, rc = O.sh_material(vs2, den2, c.h, c.dt)
    assert rc == 0
    dev = _shot(c, prec, second=(vp2, vs2, den2, mat2))
    host = _shot(c, prec, mat=c.mat, second=(vp2, vs2, den2, mat2))
    for a, b in zip(dev, host):
        np.testing.assert_array_equal(a, b)
    assert np.abs(dev[1]).max() > 0  # the wavefields (the receivers lie beyond 60 steps' reach)
