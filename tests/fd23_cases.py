"""Shared test set-up: seeded synthetic models and the matching oracle /
product configuration of one shot."""
import numpy as np

from oracle import fd23_oracle as O


def layered_model(nx, nz, seed, vmin=3.0, vmax=6.0, fluid_rows=None, nlayer=5):
    """Seeded flat layers with a small smooth lateral perturbation;
    vs = vp/1.73, rho = 0.31*vp^0.25 (km/s, g/cc style units)."""
    rng = np.random.default_rng(seed)
    bounds = np.sort(rng.integers(nz // 10, nz - 1, size=nlayer - 1))
    vel = rng.uniform(vmin, vmax, size=nlayer)
    vp = np.empty((nz, nx))
    layer = np.searchsorted(bounds, np.arange(nz), side="right")
    vp[:] = vel[layer][:, None]
    xx = np.linspace(0, 2 * np.pi, nx)
    zz = np.linspace(0, np.pi, nz)
    vp *= 1.0 + 0.03 * np.sin(3 * xx)[None, :] * np.sin(2 * zz)[:, None]
    vs = vp / 1.73
    den = 0.31 * vp ** 0.25 * 8.0
    if fluid_rows is not None:
        vs[fluid_rows[0]:fluid_rows[1], :] = 0.0
    return vp, vs, den


class Case:
    """One shot: model, CPML, point source, receivers; runs the oracle and
    configures a product Solver identically."""

    def __init__(self, wave, nx, nz, npml=12, h=0.3, dt=0.01, kind=3, seed=0, topabsorb=0,
                 nt=60, xs=None, zs=None, moment=(0.0, 20.0, 90.0, 45.0), fluid=False,
                 wavelet=("gauss", -5)):
        self.wave, self.nx, self.nz, self.npml = wave, nx, nz, npml
        self.h, self.dt, self.kind, self.topabsorb, self.nt = h, dt, kind, topabsorb, nt
        fr = (nz // 3, nz // 3 + 6) if fluid else None
        self.vp, self.vs, self.den = layered_model(nx, nz, seed, fluid_rows=fr)
        self.pml = dict(pml_dt=dt * 0.5, pml_r=1e-11, pml_v=30.0, pml_fc=2.0)
        self.xs = nx // 2 if xs is None else xs
        self.zs = nz // 4 if zs is None else zs
        if wavelet[0] == "gauss":
            self.src = O.gaussian(dt, wavelet[1])
        else:
            self.src = O.ricker(dt, wavelet[1])
        if wave == "psv":
            self.mat, self.stab, rc = O.psv_material(self.vp, self.vs, self.den, h, dt)
            self.bck = O.cpml_psv(nx, nz, npml, **_pml_args(self.pml))
            self.m = O.moment_psv(*moment)
        else:
            self.mat, self.stab, rc = O.sh_material(self.vs, self.den, h, dt)
            self.bck = O.cpml_sh(nx, nz, npml, **_pml_args(self.pml))
            self.m = O.moment_sh(*moment)
        assert rc == 0, "test model must pass the CFL check"
        self.terms = O.source_terms(wave, kind, nx, self.xs, self.zs, self.m, h, dt, self.src, nt)
        # a line of surface receivers and a buried one
        rx, rz = O.receivers_line(max(1, (nx - 10) // 7), 4, 0, 7, 0)
        rx2, rz2 = O.receivers_line(3, nx // 3, nz // 2, 5, 3)
        self.rx = np.concatenate([rx, rx2])
        self.rz = np.concatenate([rz, rz2])
        self.rx = np.clip(self.rx, 0, nx - 1)
        self.rz = np.clip(self.rz, 0, nz - 1)
        self.rec = self.rx + self.rz * nx

    def oracle(self, prec, nt=None, itrecord=1, it0=0, state=None, punch=None):
        nt = self.nt if nt is None else nt
        if self.wave == "psv":
            su, sw, st = O.psv_run(prec, self.nx, self.nz, self.npml, self.topabsorb, self.mat,
                                   self.bck, self.terms, self.rec, self.rec, nt, itrecord, it0,
                                   state, punch=punch)
            return [su, sw], st
        s, st = O.sh_run(prec, self.nx, self.nz, self.npml, self.topabsorb, self.mat, self.bck,
                         self.terms, self.rec, nt, itrecord, it0, state, punch=punch)
        return [s], st

    def straight_times(self, vmax=None):
        """Travel times t[nz, nx] along straight rays from the source at the
        fastest velocity of the model: never later than the first arrival."""
        vmax = float(self.vp.max() if self.wave == "psv" else self.vs.max()) if vmax is None else vmax
        zz, xx = np.mgrid[0:self.nz, 0:self.nx]
        return np.hypot(xx - self.xs, zz - self.zs) * self.h / vmax

    def solver(self, prec, kernel="auto"):
        import fd23_gb300 as F
        s = F.Solver(self.wave, self.nx, self.nz, self.npml, self.h, self.dt, prec=prec,
                     topabsorb=self.topabsorb, kernel=kernel, **self.pml)
        s.set_model(self.vp if self.wave == "psv" else None, self.vs, self.den)
        s.set_source(self.kind, self.xs, self.zs, self.m, self.src, self.nt)
        s.set_receivers(0, self.rx, self.rz)
        if self.wave == "psv":
            s.set_receivers(1, self.rx, self.rz)
        return s


def _pml_args(p):
    return dict(pml_dt=p["pml_dt"], pml_r=p["pml_r"], pml_v=p["pml_v"], pml_fc=p["pml_fc"])
