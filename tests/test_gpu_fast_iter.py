"""The uniform fast iterations of the single-shot 16-bit fused sweep
(fd23_gb300/csrc/fd23_fused.cuh, Cfg::FAST_ITER).

A warp takes them on rows that are z-interior in both its stress row and its
velocity row, when all of its lanes are x-interior and its item has no source
term.  The cases below move where they start and stop: no CPML (from row 4),
an absorbing top (from row npml), a source item in mid-grid (per-lane
iterations there), a grid barely wider than one strip (edge lanes in every
warp), a tall grid whose items run for dozens of blocks, and two plans whose
items start on different rows.  In every case the
fused sweep equals the two-pass sweep bit for bit, as the two round through
the same storage at the same points.
"""
import numpy as np
import pytest

from tests.fd23_cases import Case

pytestmark = pytest.mark.gpu

CASES = [
    dict(wave="psv", nx=500, nz=260, npml=0),
    dict(wave="psv", nx=500, nz=260, npml=20, topabsorb=1),
    dict(wave="psv", nx=500, nz=260, npml=12, xs=250, zs=130),
    dict(wave="psv", nx=140, nz=200, npml=8),
    # long items (one CTA per SM, a sixteenth or an eighth of a wave):
    # most iterations fast
    dict(wave="psv", nx=1000, nz=1200, npml=20, per_sm=1, ov_scale=1 / 16),
    dict(wave="sh", nx=500, nz=260, npml=0),
    dict(wave="sh", nx=500, nz=260, npml=16, topabsorb=1),
]


def _ids(c):
    return "%s_%dx%d_pml%d_top%d%s" % (c["wave"], c["nx"], c["nz"], c["npml"], c.get("topabsorb", 0),
                                       "_src_mid" if "zs" in c else "")


@pytest.mark.parametrize("oversub", [1.0, 3.0])
@pytest.mark.parametrize("prec", ["f16", "bf16", "f32"])
@pytest.mark.parametrize("cfg", CASES, ids=_ids)
def test_fast_iterations_equal_twopass(cfg, prec, oversub):
    """FP32 runs the instantiation with fast iterations (fast_iter = 1), the
    16-bit forms the one they always take."""
    F = pytest.importorskip("fd23_gb300")
    plan = {k: cfg[k] for k in ("per_sm", "ov_scale") if k in cfg}
    c = Case(nt=50, seed=21, **{k: v for k, v in cfg.items() if k not in plan})
    per_sm, ov = plan.get("per_sm", 3), oversub * plan.get("ov_scale", 1.0)

    def run(kernel):
        s = c.solver(prec, kernel)
        if kernel == "fused":
            s.set_plan(4.0, 2.5, per_sm, ov, fast_iter=int(prec == "f32"))
            assert s.plan()["fast_iter"] == int(prec == "f32")
        s.run(c.nt, 1)
        out = [s.seismograms(0)] + ([s.seismograms(1)] if c.wave == "psv" else []) + [s.get_state()]
        s.close()
        return out

    fused, twopass = run("fused"), run("twopass")
    assert np.isfinite(fused[-1]).all()
    for a, b in zip(fused, twopass):
        np.testing.assert_array_equal(a, b)


def test_fp32_autotune_tries_the_fast_instantiation():
    """The single-shot FP32 autotune times its best plan once more on the
    sweep with fast iterations (the last trial) and keeps the faster; the
    batch and 16-bit storage do not add that trial."""
    F = pytest.importorskip("fd23_gb300")
    c = Case("psv", 600, 300, npml=20, nt=40, seed=22)
    s = c.solver("f32", "fused")
    tab = s.autotune(2)
    assert tab[-1]["fast_iter"] == 1 and all(t["fast_iter"] == 0 for t in tab[:-1])
    assert s.plan()["fast_iter"] in (0, 1)
    with pytest.raises(F.Fd23Error):
        s.set_plan(4.0, 2.5, 3, 1.0, fast_iter=2)  # 0 or 1 only
    s.run(c.nt, 1)
    seis, st = c.oracle("f32")
    np.testing.assert_array_equal(s.get_state(), st)
    s.close()
    h = c.solver("f16", "fused")
    assert all(t["fast_iter"] == 0 for t in h.autotune(2))
    h.close()
