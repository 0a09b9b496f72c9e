"""Benchmark: P-SV time stepping on GB300, cell-updates per second.

Workload (one bench "step" = one whole shot from a zero wavefield):
  P-SV, nx=4000, nz=2000, h=5 m, dt=4e-4 s, 5000 time steps; 12 seeded flat
  layers with vp ~ U[1500, 4500] m/s plus a seeded Gaussian-smoothed 5 %
  perturbation, vs = vp/1.73, rho = 310 vp^0.25; 15 Hz Ricker explosion;
  40-cell CPML; 400 surface stations recorded as 800 traces per component.
  Synthetic data (the reference publishes no data set for this path).

value: cell-updates/s with the model already resident in HBM (CUDA events on
       the solver's stream around K whole shots).
e2e:   the same metric through the public API with host buffers in pinned
       memory: model upload + material build, the shot, device->host
       seismograms into caller-owned buffers.
roofline: the fused sweep kernel against the measured HBM copy bandwidth.
cpu_baseline: the oracle's restatement of the reference update loop on the
       host cores, on a bounded sample of the same grid.

Hybrid-box workload (--config c2): the same model and grid, 3000 steps,
  a 2000 x 1000 box at (1000, 10) around the source with 4-cell add and sub
  rings.  The incident field on the ring cells (U, W, Txx, Txz, Tzz every
  step, 2.9 GB FP32) is recorded from a plain run of the same shot; the box
  run has no point source.  Its surface seismograms must equal the recorded
  run's bit for bit ("check" in the output line).

SH workload (--config c0): 800 x 400 SH grid, h=10 m, dt=1e-3 s, 2000 steps,
  two layers (vs 2000 / 3000 m/s, rho 2200 / 2500, interface at iz=200),
  10 Hz Ricker line force on V at (400, 20), 20-cell CPML, free surface, 200
  surface receivers.  The 10 MB working set stays in L2 within a shot, so the
  step is launch- and latency-bound; the run is the fused sweep captured in a
  CUDA graph (a one-shot batch), or with --kernel persist one cooperative
  launch per shot (grid barriers between the update phases).  L2 is flushed
  between timed shots.

Batched workload (--config c4): 64 shots with seeded grid sizes nx in
  [1000, 4000], nz in [500, 2000] (not tile multiples), h=5 m, dt=4e-4 s,
  3000 steps, per-shot seeded layered models, Ricker 8-25 Hz explosions,
  40-cell CPML, 200 stations (400 traces) per component.  All shots advance
  in one sweep launch per step (a CUDA graph per run); the work plan is
  autotuned first (not timed).  The line also carries the same shots run one
  by one with the plain FP32 solver, and for 16-bit storage the seismogram
  relative-L2 error against FP64 runs of a seeded subset of the shots.

Windowed workload (--config c5, usepunch): the C1 shot with tile step
  windows (32 x 16 tiles) from straight-ray travel times at the fastest
  velocity, opening 0.02 s before that time and not closing within the run;
  18.5 % of the tile-steps are live.  value counts every cell of the grid
  per step (the run advances the whole grid); the roofline counts the bytes
  of the live tiles only; accuracy carries the seismogram error against the
  same shot without windows.

Generated-box workload (--config c6, the reference's hybrid use): the C1
  grid and model, 5000 steps, a 32 x 32 box around a line moment source
  buried at (2000, 200) (strike 30, dip 60, rake 90, one-sided Gaussian
  alpha = -20); the box material is the source cell's vp, vs, rho (box
  cells of the model replaced, as the reference does); the incident field
  is generated on the device every shot (the box-source generator: FP64
  Green's functions and wavelet convolution on the ring stencils, then the
  setboxsource step).  "check" compares a shot against the same shot driven
  through the host path (generator planes -> setboxsource on the host ->
  incident upload) bit for bit.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config c0|c1|c2|c3|c4|c5|c6] [--nt NT] [--prec f32|bf16|f16|f64]
                  [--kernel fused|twopass]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NX, NZ, H, DT, NT, NPML, F0 = 4000, 2000, 5.0, 4e-4, 5000, 40, 15.0
NSTA = 400
# hybrid-box workload: box origin and size, steps
BOX_X0, BOX_Z0, BOX_BX, BOX_BZ, NT_BOX = 1000, 10, 2000, 1000, 3000
# generated-box workload: source cell, box width, mechanism, Gaussian alpha
LB_XS, LB_ZS, LB_BW, LB_MECH, LB_ALPHA = NX // 2, 200, 32, (30.0, 60.0, 90.0, 0.0), -20
# batched workload: shots, steps, stations per shot, shots checked against FP64
NSHOT_B, NT_B, NSTA_B, NCHECK_B = 64, 3000, 200, 6


def c1_model(nx=NX, nz=NZ, seed=1):
    rng = np.random.default_rng(seed)
    bounds = np.sort(rng.choice(np.arange(nz // 20, nz - nz // 20), size=11, replace=False))
    vel = rng.uniform(1500.0, 4500.0, size=12)
    layer = np.searchsorted(bounds, np.arange(nz), side="right")
    vp = np.repeat(vel[layer][:, None], nx, axis=1)
    noise = rng.standard_normal((nz, nx))
    kz = np.fft.fftfreq(nz)[:, None]
    kx = np.fft.rfftfreq(nx)[None, :]
    sig = 20.0
    smooth = np.fft.irfft2(np.fft.rfft2(noise) * np.exp(-2 * (np.pi * sig) ** 2 * (kx ** 2 + kz ** 2)),
                           s=(nz, nx))
    smooth *= 0.05 / np.abs(smooth).max()
    vp *= 1.0 + smooth
    vs = vp / 1.73
    rho = 310.0 * vp ** 0.25
    return vp, vs, rho


PUNCH_BEFORE, PUNCH_AFTER = 0.02, 10.0
# block weights (x-CPML, z-CPML) of the windowed workload's phase plans
C5_PLAN = (6.0, 4.0)


def punch_windows_c5(vp):
    """Tile step windows of the windowed C1 workload: straight-ray travel
    times from the source at the fastest velocity, opening PUNCH_BEFORE
    seconds early and closing PUNCH_AFTER seconds late (after the run)."""
    import fd23_gb300 as F
    zz, xx = np.mgrid[0:NZ, 0:NX]
    t = np.hypot(xx - NX // 2, zz - 20) * H / float(vp.max())
    return F.punch_windows(t, PUNCH_BEFORE, PUNCH_AFTER, DT, "f64")


def punch_active_fraction(first, last, nt):
    """Mean fraction of tiles the sweep must touch per step: tiles not steady
    (updated at this step or the last)."""
    f = np.asarray(first, np.int64)[:, None]
    l = np.asarray(last, np.int64)[:, None]
    it = np.arange(nt)[None, :]
    live = (f < it) & (it <= l) & (l - f >= 2)
    return float(live.mean())


def alg_bytes(nx, nz, npml, es, topabsorb=0):
    """Compulsory HBM bytes of one time step: every wavefield read and written
    once and every material array read once (5+5 arrays of es bytes), plus the
    CPML memory variables (4 per PML cell, read and written, FP32/FP64)."""
    cs = 8 if es == 8 else 4
    npml_cells = 2 * npml * nz + npml * nx * (1 + topabsorb)
    return (5 * 2 + 5) * es * nx * nz + 4 * 2 * cs * npml_cells


def box_alg_bytes(bx, bz, nring, es):
    """Compulsory HBM bytes the box adds to one step: the residual stress
    update (read U W Txx Txz Tzz LAM MU MUA, write Txx Txz Tzz) and velocity
    update (read Txx Txz Tzz U W BU BW, write U W) on the (bx-8)(bz-8)
    interior cells, and per ring cell the incident field (5 values) and the
    exchange (read r or g, write g or r, for 5 fields)."""
    return 20 * es * (bx - 8) * (bz - 8) + 15 * es * nring


def pinned_copy(torch, a):
    """a copied into page-locked host memory (a numpy view of it)."""
    t = torch.empty(a.shape, dtype=torch.from_numpy(np.empty(0, a.dtype)).dtype, pin_memory=True)
    out = t.numpy()
    out[...] = a
    return out


def pinned_like(torch, a):
    """A zeroed page-locked host array of a's shape and type."""
    return pinned_copy(torch, np.zeros_like(a))


def max_over_ranks(ms, dist):
    """Slowest rank's time (replicas run independent shots; the job's time is
    the slowest one's)."""
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64)
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(budget_s=15.0, threads=0):
    """Oracle restatement of the reference update loop (FP32, all host
    threads) on the benchmark grid for as many steps as fit the budget."""
    from oracle import fd23_oracle as O
    vp, vs, rho = c1_model(NX, NZ)
    mat, _, _ = O.psv_material(vp, vs, rho, H, DT)
    bck = O.cpml_psv(NX, NZ, NPML, DT, 1e-11, vp.max() / H, F0)
    src = O.ricker(DT, F0)
    terms = O.source_terms("psv", 1, NX, NX // 2, 20, np.array([1.0, 0, 1.0]), H, DT, src, NT)
    rec = np.arange(200, 200 + 9 * NSTA, 9)
    # a short run to size the sample (the first steps also pay for thread
    # start-up and first touch), then one contiguous run that fits the budget
    O.psv_run("f32", NX, NZ, NPML, 0, mat, bck, terms, rec, rec + NX, 1, nthreads=threads)
    t0 = time.perf_counter()
    O.psv_run("f32", NX, NZ, NPML, 0, mat, bck, terms, rec, rec + NX, 16, nthreads=threads)
    one = (time.perf_counter() - t0) / 16
    steps = int(max(3, min(NT, budget_s / max(one, 1e-4))))
    t0 = time.perf_counter()
    O.psv_run("f32", NX, NZ, NPML, 0, mat, bck, terms, rec, rec + NX, steps, nthreads=threads)
    t_used = time.perf_counter() - t0
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    return {"value": NX * NZ * steps / t_used, "unit": "cell-updates/s", "cores": cores,
            "kind": "port",
            "sample": "%d steps of the %dx%d grid (%.1f s), FP32 oracle, %d threads" % (
                steps, NX, NZ, t_used, cores)}


def run_reference_arm(args, rank, world):
    """The reference's update loop on the host cores (the oracle's restatement,
    FP32, every host thread).  One bench step = a bounded sample of the shot:
    m consecutive time steps of the full grid, m sized to about 8 s; warm-up
    steps run one time step each."""
    if rank != 0:
        return
    from oracle import fd23_oracle as O
    vp, vs, rho = c1_model()
    mat, _, _ = O.psv_material(vp, vs, rho, H, DT)
    bck = O.cpml_psv(NX, NZ, NPML, DT, 1e-11, vp.max() / H, F0)
    src = O.ricker(DT, F0)
    terms = O.source_terms("psv", 1, NX, NX // 2, 20, np.array([1.0, 0, 1.0]), H, DT, src, NT)
    rec = np.arange(200, 200 + 9 * NSTA, 9)
    state, it = None, 0
    for _ in range(max(args.warmup, 1)):
        _, _, state = O.psv_run("f32", NX, NZ, NPML, 0, mat, bck, terms, rec, rec + NX, 1, it0=it,
                                state=state)
        it += 1
    t0 = time.perf_counter()
    _, _, state = O.psv_run("f32", NX, NZ, NPML, 0, mat, bck, terms, rec, rec + NX, 2, it0=it,
                            state=state)
    it += 2
    m = int(max(2, min(NT // 4, 8.0 / max((time.perf_counter() - t0) / 2, 1e-4))))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, _, state = O.psv_run("f32", NX, NZ, NPML, 0, mat, bck, terms, rec, rec + NX, m, it0=it,
                                state=state)
        it += m
    t = time.perf_counter() - t0
    value = NX * NZ * m * args.steps / t
    cores = os.cpu_count() or 1
    cb = {"value": value, "unit": "cell-updates/s", "cores": cores, "kind": "port",
          "sample": "%d samples of %d consecutive time steps of the %dx%d grid (%.1f s), FP32 "
                    "oracle restatement of the reference update loop, %d threads" % (
                        args.steps, m, NX, NZ, t, cores)}
    sample_ms = t / args.steps * 1e3
    line = {"impl": "reference", "metric": "cell-updates/s", "value": value,
            "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sample_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "psv_%dx%d_%dsteps_c1" % (NX, NZ, NT), "nx": NX, "nz": NZ, "nt": NT,
                       "h_m": H, "dt_s": DT, "npml": NPML, "source": "15 Hz Ricker explosion",
                       "traces": 4 * NSTA, "prec": "f32",
                       "parallelism": "host cores x%d" % cores},
            "note": "one bench step = one sample of %d consecutive time steps of the shot "
                    "(ms_per_step is that sample's measured time); shot_ms_extrapolated = one "
                    "whole %d-step shot at the measured rate.  The reference's own sources are "
                    "not on the GPU host, so its update loop runs as the oracle restatement" % (m, NT),
            "shot_ms_extrapolated": NX * NZ * NT / value * 1e3,
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    global NX, NZ, H, DT, NT
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours")
    ap.add_argument("--nt", type=int, default=NT)
    ap.add_argument("--prec", default="f32")
    ap.add_argument("--kernel", default=None, choices=["fused", "twopass", "persist", "fused2"],
                    help="default fused; persist: a run in one cooperative launch (small grids); "
                         "fused2: two time steps per launch (P-SV FP32)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--bands", type=int, choices=(0, 1), default=None,
                    help="with --no-tune: the default block weights, cut strip after strip (0) or banded (1)")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--config", default="c1", choices=["c0", "c1", "c2", "c3", "c4", "c5", "c6"])
    ap.add_argument("--plan", default=None, type=lambda v: tuple(float(x) for x in v.split(",")),
                    help="c5: x-CPML,z-CPML block weights of the phase plans")
    args = ap.parse_args()
    if args.kernel is None:
        args.kernel = "fused"
    if args.config == "c3":
        # the large grid: 16000 x 8000, h 2.5 m, dt 2e-4 s, 8000 steps, C1-style model
        NX, NZ, H, DT, NT = 16000, 8000, 2.5, 2e-4, 8000
        args.nt = min(args.nt, NT) if args.nt != 5000 else NT
        args.no_accuracy = True  # an FP64 run of this grid takes minutes

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch
    import fd23_gb300 as F
    torch.cuda.set_device(local)
    if args.config == "c2":
        bench_box(args, F, torch, rank, world, local, dist)
        return
    if args.config == "c4":
        bench_batch(args, F, torch, rank, world, local, dist)
        return
    if args.config == "c6":
        bench_linebox(args, F, torch, rank, world, local, dist)
        return
    if args.config == "c0":
        bench_sh(args, F, torch, rank, world, local, dist)
        return
    nt = args.nt
    vp, vs, rho = c1_model(NX, NZ, seed=1 + rank)
    pml_v = float(vp.max()) / H
    s = F.Solver("psv", NX, NZ, NPML, H, DT, prec=args.prec, pml_dt=DT, pml_v=pml_v, pml_r=1e-11,
                 pml_fc=F0, device=local, kernel=args.kernel)
    s.set_model(vp, vs, rho)
    src = F.wavelet_ricker(DT, F0)
    s.set_source(F.SRC_EXPLOSION, NX // 2, 20, None, src, nt)
    rxu, rzu = F.receivers_line(NSTA, 200, 0, 9, 0)
    rxw, rzw = F.receivers_line(NSTA, 200, 1, 9, 0)
    s.set_receivers(0, rxu, rzu)
    s.set_receivers(1, rxw, rzw)
    stream = torch.cuda.ExternalStream(s.stream, device=local)
    # work plan picked by the autotuner on this shot (set-up, not timed)
    tune = s.autotune(10) if args.kernel == "fused" and not args.no_tune and args.config != "c5" else []
    best_plan = s.plan() if tune else None  # the plan the autotuner kept
    if args.kernel in ("fused", "fused2") and args.no_tune and args.bands is not None and args.config != "c5":
        s.set_plan(4.0, 3.0, 3, 1.0, bands=args.bands)
        best_plan = s.plan()
    punch = None
    if args.config == "c5":
        # usepunch: tile step windows from straight-ray travel times at the
        # fastest velocity (never later than the first arrival), opening
        # PUNCH_BEFORE early and not closing within the run.  The sweep plans
        # every 128-step phase over the blocks live in it, one wave of CTAs
        # with the C1 block weights.
        first, last = punch_windows_c5(vp)
        s.set_punch(first, last)
        if args.kernel == "fused":
            wx, wz = C5_PLAN if args.plan is None else args.plan
            s.set_plan(wx, wz, 3, 1.0)
            best_plan = {"wx": wx, "wz": wz, "oversub": 1.0, "phase_steps": 128}
        punch = {"first": first, "last": last, "active": punch_active_fraction(first, last, nt)}

    def shot():
        s.reset()
        s.run(nt, 1)

    for _ in range(args.warmup):
        shot()
    s.sync()
    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        shot()
    e1.record(stream)
    s.sync()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop() if rank == 0 else None
    ms_max = max_over_ranks(ms, dist)
    cells = NX * NZ * nt * args.steps * world
    value = cells / (ms_max * 1e-3)
    seis = (s.seismograms(0), s.seismograms(1))

    # c5: the same shot without windows, same precision (what the windows change)
    punch_vs_plain = None
    if punch is not None and rank == 0 and not args.no_accuracy:
        r = F.Solver("psv", NX, NZ, NPML, H, DT, prec=args.prec, pml_dt=DT, pml_v=pml_v, pml_r=1e-11, pml_fc=F0,
                     device=local, kernel=args.kernel)
        r.set_model(vp, vs, rho)
        r.set_source(F.SRC_EXPLOSION, NX // 2, 20, None, src, nt)
        r.set_receivers(0, rxu, rzu)
        r.set_receivers(1, rxw, rzw)
        r.run(nt, 1)
        ref = np.concatenate([r.seismograms(0).ravel(), r.seismograms(1).ravel()]).astype(np.float64)
        got = np.concatenate([seis[0].ravel(), seis[1].ravel()]).astype(np.float64)
        punch_vs_plain = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        r.close()

    # seismogram error against an FP64 run of the same shot (GPU FP64 sweep,
    # bit-identical to the FP64 oracle)
    accuracy = None
    if rank == 0 and args.prec != "f64" and not args.no_accuracy:
        r = F.Solver("psv", NX, NZ, NPML, H, DT, prec="f64", pml_dt=DT, pml_v=pml_v, pml_r=1e-11, pml_fc=F0,
                     device=local, kernel="fused")
        r.set_model(vp, vs, rho)
        r.set_source(F.SRC_EXPLOSION, NX // 2, 20, None, src, nt)
        r.set_receivers(0, rxu, rzu)
        r.set_receivers(1, rxw, rzw)
        r.run(nt, 1)
        ref = np.concatenate([r.seismograms(0).ravel(), r.seismograms(1).ravel()])
        got = np.concatenate([seis[0].ravel(), seis[1].ravel()]).astype(np.float64)
        accuracy = {"seismogram_rel_l2_vs_fp64": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
                    "traces": int(seis[0].shape[1] + seis[1].shape[1]), "steps": nt}
        r.close()

    # end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        es = {"f32": 4, "f64": 8, "bf16": 2, "f16": 2}[args.prec]
        cs = 8 if args.prec == "f64" else 4
        # inputs and results in pinned host memory (set up before the timed shots)
        hvp, hvs, hrho = (pinned_copy(torch, a) for a in (vp, vs, rho))
        hsu, hsw = (pinned_like(torch, s.seismograms(f)) for f in (0, 1))
        times = []
        seis_bytes = 0
        for _ in range(max(1, min(args.steps, 2))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.set_model(hvp, hvs, hrho)
            shot()
            su, sw = s.seismograms(0, hsu), s.seismograms(1, hsw)
            times.append(time.perf_counter() - t0)
            seis_bytes = su.nbytes + sw.nbytes
        # vp, vs, rho go up as doubles; the material is built (and for the
        # 16-bit forms scaled and rounded) on the device
        model_bytes = 3 * NX * NZ * 8
        e2e = {"value": NX * NZ * nt / statistics.mean(times) * world, "unit": "cell-updates/s",
               "h2d_bytes_per_step": model_bytes + 2 * nt * cs,
               "d2h_bytes_per_step": seis_bytes}

    hbm, peak_kind = load_peaks()
    es = {"f32": 4, "f64": 8, "bf16": 2, "f16": 2}[args.prec]
    # the two-step sweep advances two steps per launch and moves the same
    # compulsory bytes per launch (each field read and written once, the
    # material and the memory variables once) as a one-step launch
    launches = nt // 2 + nt % 2 if args.kernel == "fused2" else nt
    per_launch_ms = ms_max / (args.steps * launches)
    ab = alg_bytes(NX, NZ, NPML, es)
    if punch is not None:
        ab = ab * punch["active"]  # only the cells of tiles the windows leave live move
    achieved = ab / (per_launch_ms * 1e-3) / 1e9
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic_per_cell.json")
    if os.path.exists(tfile):
        key = "%s_psv_%s" % ("fused2" if args.kernel == "fused2" else "fused", args.prec)
        if best_plan and best_plan.get("bands"):
            key += "_bands1"  # the banded plan re-reads less (shared halo lines hit in L2)
        tb = json.load(open(tfile)).get(key)
        if tb:
            traffic = tb * NX * NZ
    line = {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.prec,
            "data": "synthetic",
            "config": {"workload": "psv_%dx%d_%dsteps_%s" % (NX, NZ, NT, args.config), "nx": NX, "nz": NZ,
                       "nt": nt,
                       "h_m": H, "dt_s": DT, "npml": NPML, "source": "15 Hz Ricker explosion",
                       "traces": 4 * NSTA, "kernel": args.kernel, "prec": args.prec,
                       "l2": "inputs larger than L2 (%.0f MB resident)" % (
                           (15 * es) * NX * NZ / 1e6),
                       "parallelism": "replicas x%d" % world},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic,
                         "peak_source": peak_kind,
                         "alg_bytes_per_launch": ab,
                         "launch_ms": per_launch_ms},
            "gpu_launches": args.steps * (launches + 1),
            "clocks": clocks,
            "e2e": e2e}
    if best_plan:
        line["config"]["plan"] = {"wx": best_plan["wx"], "wz": best_plan["wz"], "oversub": best_plan["oversub"],
                                  "bands": best_plan.get("bands", 0), "fast_iter": best_plan.get("fast_iter", 0),
                                  "autotune_trials": len(tune)}
        if tune:
            # fastest trial of each way of cutting (ms per step); FP32: the
            # best plan on the sweep with uniform fast iterations
            line["config"]["plan"]["best_trial_ms"] = {
                "bands%d" % b: min((t["ms_per_step"] for t in tune if t["bands"] == b and not t["fast_iter"]),
                                   default=None)
                for b in (0, 1)}
            fast = [t["ms_per_step"] for t in tune if t["fast_iter"]]
            if fast:
                line["config"]["plan"]["best_trial_ms"]["fast_iter1"] = min(fast)
    if accuracy:
        line["accuracy"] = accuracy
    if punch is not None:
        line["config"]["usepunch"] = {"tiles": "32x16", "before_s": PUNCH_BEFORE, "after_s": PUNCH_AFTER,
                                      "travel_times": "straight rays at the fastest velocity",
                                      "tile_steps_live_fraction": punch["active"]}
        line.setdefault("accuracy", {})["seismogram_rel_l2_vs_same_shot_without_windows"] = punch_vs_plain
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line), flush=True)
    s.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def cpu_baseline_box(inc, budget_s=15.0, threads=0):
    """Oracle box run (FP32, all host threads) on the benchmark grid for as
    many steps as fit the budget, driven by the first steps of the recorded
    incident field."""
    from oracle import fd23_oracle as O
    vp, vs, rho = c1_model()
    mat, _, _ = O.psv_material(vp, vs, rho, H, DT)
    bck = O.cpml_psv(NX, NZ, NPML, DT, 1e-11, vp.max() / H, F0)
    box = (BOX_X0, BOX_Z0, BOX_BX, BOX_BZ)
    rmat = np.ascontiguousarray(mat[:, BOX_Z0:BOX_Z0 + BOX_BZ, BOX_X0:BOX_X0 + BOX_BX])
    none = (np.zeros(0, np.int32), np.zeros(0, np.int64), np.zeros((0, 1)))
    rf = np.zeros(NSTA, np.int32)
    ri = np.arange(200, 200 + 9 * NSTA, 9).astype(np.int64)
    O.psv_box_run("f32", NX, NZ, NPML, 0, mat, bck, none, rf, ri, 1, box, rmat, inc[:1],
                  nthreads=threads)
    t0 = time.perf_counter()
    O.psv_box_run("f32", NX, NZ, NPML, 0, mat, bck, none, rf, ri, 16, box, rmat, inc[:16],
                  nthreads=threads)
    one = (time.perf_counter() - t0) / 16
    steps = int(max(4, min(budget_s / max(one, 1e-4), inc.shape[0])))
    t0 = time.perf_counter()
    O.psv_box_run("f32", NX, NZ, NPML, 0, mat, bck, none, rf, ri, steps, box, rmat, inc[:steps],
                  nthreads=threads)
    t_used = time.perf_counter() - t0
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    return {"value": NX * NZ * steps / t_used, "unit": "cell-updates/s", "cores": cores,
            "kind": "port",
            "sample": "%d box steps of the %dx%d grid with the %dx%d box (%.1f s), FP32 oracle, "
                      "%d threads" % (steps, NX, NZ, BOX_BX, BOX_BZ, t_used, cores)}


def bench_box(args, F, torch, rank, world, local, dist):
    """Hybrid-box workload: record the ring field of a plain run, then time box
    runs driven by it."""
    nt = min(args.nt, NT_BOX)
    vp, vs, rho = c1_model(seed=1 + rank)
    pml_v = float(vp.max()) / H
    kw = dict(prec="f32", pml_dt=DT, pml_v=pml_v, pml_r=1e-11, pml_fc=F0, device=local,
              kernel=args.kernel)
    src = F.wavelet_ricker(DT, F0)
    rxu, rzu = F.receivers_line(NSTA, 200, 0, 9, 0)
    rxw, rzw = F.receivers_line(NSTA, 200, 1, 9, 0)
    rix, riz = F.box_ring_cells(BOX_X0, BOX_Z0, BOX_BX, BOX_BZ)
    nring = len(rix)
    # 1. the recorded run: point source, surface lines + every ring cell
    p = F.Solver("psv", NX, NZ, NPML, H, DT, **kw)
    p.set_model(vp, vs, rho)
    p.set_source(F.SRC_EXPLOSION, NX // 2, 20, None, src, nt)
    lines = {0: (rxu, rzu), 1: (rxw, rzw)}
    for f in range(5):
        lx, lz = lines.get(f, (np.zeros(0, np.int32), np.zeros(0, np.int32)))
        p.set_receivers(f, np.concatenate([lx, rix]), np.concatenate([lz, riz]))
    p.run(nt, 1)
    nl = len(rxu)
    inc = torch.empty((nt, 5, nring), dtype=torch.float32, pin_memory=True).numpy()
    ref_traces = {}
    for f in range(5):
        sg = p.seismograms(f)
        k = nl if f < 2 else 0
        if f < 2:
            ref_traces[f] = sg[:, :nl].copy()
            inc[0, f] = 0.0
            inc[1:, f] = sg[:-1, k:]   # velocities before the step
        else:
            inc[:, f] = sg[:, k:]      # stresses after the step's stress update
        del sg
    p.close()
    # 2. the box solver: no point source
    s = F.Solver("psv", NX, NZ, NPML, H, DT, **kw)
    s.set_model(vp, vs, rho)
    s.set_receivers(0, rxu, rzu)
    s.set_receivers(1, rxw, rzw)
    s.set_box(BOX_X0, BOX_Z0, BOX_BX, BOX_BZ)
    s.set_box_incident(inc, 0)
    stream = torch.cuda.ExternalStream(s.stream, device=local)

    def shot():
        s.reset()
        s.run(nt, 1)

    for _ in range(args.warmup):
        shot()
    check = bool(np.array_equal(s.seismograms(0), ref_traces[0]) and
                 np.array_equal(s.seismograms(1), ref_traces[1]))
    s.sync()
    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        shot()
    e1.record(stream)
    s.sync()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop() if rank == 0 else None
    ms_max = max_over_ranks(ms, dist)
    value = NX * NZ * nt * args.steps * world / (ms_max * 1e-3)

    e2e = None
    if not args.no_e2e:
        hvp, hvs, hrho = (pinned_copy(torch, a) for a in (vp, vs, rho))
        hsu, hsw = (pinned_like(torch, s.seismograms(f)) for f in (0, 1))
        times, parts = [], []
        seis_bytes = 0
        for _ in range(max(1, min(args.steps, 2))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.set_model(hvp, hvs, hrho)
            t1 = time.perf_counter()
            s.set_box(BOX_X0, BOX_Z0, BOX_BX, BOX_BZ)
            t2 = time.perf_counter()
            s.set_box_incident(inc, 0, wait=False)  # the upload overlaps the run
            t3 = time.perf_counter()
            shot()
            su, sw = s.seismograms(0, hsu), s.seismograms(1, hsw)
            t4 = time.perf_counter()
            times.append(t4 - t0)
            # host-side milliseconds of each call (the run's launches are asynchronous:
            # its time lands in the seismogram read that waits for it)
            parts.append({"set_model": round((t1 - t0) * 1e3, 1), "set_box": round((t2 - t1) * 1e3, 1),
                          "set_box_incident_async": round((t3 - t2) * 1e3, 1),
                          "upload_run_and_read": round((t4 - t3) * 1e3, 1)})
            seis_bytes = su.nbytes + sw.nbytes
        e2e = {"value": NX * NZ * nt / statistics.mean(times) * world, "unit": "cell-updates/s",
               "h2d_bytes_per_step": 3 * NX * NZ * 8 + inc.nbytes, "d2h_bytes_per_step": seis_bytes,
               "shot_ms": [round(t * 1e3, 1) for t in times], "parts_ms": parts,
               "note": "per step = one whole box shot; the incident field is uploaded from pinned "
                       "host memory inside the timed region, on a copy stream that overlaps the run "
                       "(fd23_set_box_incident_async)"}
    hbm, peak_kind = load_peaks()
    per_step_ms = ms_max / (args.steps * nt)
    ab = alg_bytes(NX, NZ, NPML, 4) + box_alg_bytes(BOX_BX, BOX_BZ, nring, 4)
    achieved = ab / (per_step_ms * 1e-3) / 1e9
    line = {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "psv_4000x2000_3000steps_box2000x1000_c2", "nx": NX, "nz": NZ,
                       "nt": nt, "box": [BOX_X0, BOX_Z0, BOX_BX, BOX_BZ], "ring_cells": nring,
                       "incident_bytes": inc.nbytes, "kernel": args.kernel,
                       "cells_counted": "grid cells nx*nz per step (the box's residual field is "
                                        "extra work)",
                       "l2": "inputs larger than L2", "parallelism": "replicas x%d" % world},
            "check": {"surface_traces_bit_exact_vs_recorded_run": check},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": None, "peak_source": peak_kind,
                         "scope": "whole step: sweep + box kernels",
                         "alg_bytes_per_launch": ab, "launch_ms": per_step_ms},
            "gpu_launches": args.steps * nt * 4,
            "clocks": clocks,
            "e2e": e2e}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_box(inc)
    if rank == 0:
        print(json.dumps(line), flush=True)
    s.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def linebox_setup(F, vp, vs, rho):
    """Material, box and line source of the generated-box workload, built as
    the reference's PD program builds them (MATERIAL::get_model, then
    BOX::init_box homogenises the box): FP64 on the host."""
    mat, stab, rc = F.build_material("psv", vp, vs, rho, H, DT)
    if rc:
        raise RuntimeError("generated-box model fails the CFL check (stab %.3f)" % stab)
    sv = (float(vp[LB_ZS, LB_XS]), float(vs[LB_ZS, LB_XS]), float(rho[LB_ZS, LB_XS]))
    x0 = LB_XS + (LB_BW + 1) // 2 + 1 - LB_BW
    z0 = LB_ZS + (LB_BW + 1) // 2 + 1 - LB_BW
    mat, bmat, _ = F.box_material(mat, x0, z0, LB_BW, LB_BW, sv[0], sv[1], sv[2], DT, H)
    o = F.line_plane_origin(LB_BW)
    desc = F.line_desc(LB_BW + 8, LB_BW + 8, o, o, H, DT, sv[0], sv[1], sv[2], F.line_source_coefs(*LB_MECH))
    return mat, bmat, (x0, z0, LB_BW, LB_BW), desc, sv


def cpu_baseline_linebox(budget_s=15.0):
    """The generated-box shot on the host cores: the oracle's generator for the
    box planes, setboxsource, and the oracle's box run (FP32, all threads),
    for as many steps as fit the budget."""
    import fd23_gb300 as F
    from oracle import fd23_oracle as O
    vp, vs, rho = c1_model()
    mat, bmat, box, desc, sv = linebox_setup(F, vp, vs, rho)
    bck = O.cpml_psv(NX, NZ, NPML, DT, 1e-11, vp.max() / H, F0)
    none = (np.zeros(0, np.int32), np.zeros(0, np.int64), np.zeros((0, 1)))
    rf = np.zeros(NSTA, np.int32)
    ri = np.arange(200, 200 + 9 * NSTA, 9).astype(np.int64)
    src = O.gaussian(DT, LB_ALPHA)
    a = O.line_source_coefs(*LB_MECH)

    def run(steps):
        t0 = time.perf_counter()
        pl = O.line_source_planes(desc.px, desc.pz, desc.ox, desc.oz, H, DT, sv[0], sv[1], sv[2], a, src, 0,
                                  steps + 1)
        inc = np.stack([O.box_incident_from_displacement(LB_BW, LB_BW, DT, bmat, pl[i, 0], pl[i, 1], pl[i + 1, 0],
                                                         pl[i + 1, 1]) for i in range(steps)])
        O.psv_box_run("f32", NX, NZ, NPML, 0, mat, bck, none, rf, ri, steps, box, bmat, inc)
        return time.perf_counter() - t0

    one = run(8) / 8
    steps = int(max(4, min(budget_s / max(one, 1e-4), NT)))
    t_used = run(steps)
    cores = os.cpu_count() or 1
    return {"value": NX * NZ * steps / t_used, "unit": "cell-updates/s", "cores": cores, "kind": "port",
            "sample": "%d steps of the %dx%d grid with the %d-cell generated box (%.1f s): oracle generator + "
                      "setboxsource + FP32 oracle box run, %d threads" % (steps, NX, NZ, LB_BW, t_used, cores)}


def bench_linebox(args, F, torch, rank, world, local, dist):
    """Generated-box workload: the box's incident field generated on the device
    inside every timed shot."""
    nt = args.nt
    vp, vs, rho = c1_model(seed=1 + rank)
    mat, bmat, box, desc, sv = linebox_setup(F, vp, vs, rho)
    src = F.wavelet_gaussian(DT, LB_ALPHA)
    s = F.Solver("psv", NX, NZ, NPML, H, DT, prec="f32", pml_dt=DT, pml_v=float(vp.max()) / H, pml_r=1e-11,
                 pml_fc=F0, device=local, kernel=args.kernel)
    rxu, rzu = F.receivers_line(NSTA, 200, 0, 9, 0)
    rxw, rzw = F.receivers_line(NSTA, 200, 1, 9, 0)

    def configure():
        s.set_material(mat)
        s.set_receivers(0, rxu, rzu)
        s.set_receivers(1, rxw, rzw)
        s.set_box(*box, bmat=bmat)

    configure()
    nring = sum(F.box_ring_size(LB_BW, LB_BW))
    stream = torch.cuda.ExternalStream(s.stream, device=local)

    def shot():
        s.reset()
        s.set_box_line_source(desc, src, bmat, 0, nt)
        s.run(nt, 1)

    for _ in range(args.warmup):
        shot()
    got = s.seismograms(0), s.seismograms(1)
    # the same shot through the host path: generator planes, setboxsource on
    # the host, incident upload
    planes = F.line_source_planes(desc, src, 0, nt + 1, device=local)
    inc = np.stack([F.box_incident_from_displacement(LB_BW, LB_BW, DT, bmat, planes[i, 0], planes[i, 1],
                                                     planes[i + 1, 0], planes[i + 1, 1]) for i in range(nt)])
    s.reset()
    s.set_box_incident(inc.astype(np.float32), 0)
    s.run(nt, 1)
    check = bool(np.array_equal(s.seismograms(0), got[0]) and np.array_equal(s.seismograms(1), got[1]))
    reached = float(np.abs(got[0]).max())
    del planes, inc
    # the generator alone (CUDA events on the solver's stream)
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    s.set_box_line_source(desc, src, bmat, 0, nt)
    g1.record(stream)
    s.sync()
    gen_ms = g0.elapsed_time(g1)
    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        shot()
    e1.record(stream)
    s.sync()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop() if rank == 0 else None
    ms_max = max_over_ranks(ms, dist)
    value = NX * NZ * nt * args.steps * world / (ms_max * 1e-3)

    e2e = None
    if not args.no_e2e:
        hsu, hsw = (pinned_like(torch, s.seismograms(f)) for f in (0, 1))
        hvp, hvs, hrho = (pinned_copy(torch, a) for a in (vp, vs, rho))
        times = []
        seis_bytes = 0
        for _ in range(max(1, min(args.steps, 2))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            # material and the box's homogenisation and material on the device
            _, b2 = s.set_model_box(hvp, hvs, hrho, *box, *sv)
            s.reset()
            s.set_box_line_source(desc, src, b2, 0, nt)
            s.run(nt, 1)
            su, sw = s.seismograms(0, hsu), s.seismograms(1, hsw)
            times.append(time.perf_counter() - t0)
            seis_bytes = su.nbytes + sw.nbytes
        e2e = {"value": NX * NZ * nt / statistics.mean(times) * world, "unit": "cell-updates/s",
               "h2d_bytes_per_step": hvp.nbytes + hvs.nbytes + hrho.nbytes + bmat.nbytes + src.nbytes,
               "d2h_bytes_per_step": seis_bytes + bmat.nbytes,
               "shot_ms": [round(t * 1e3, 1) for t in times],
               "note": "per step = one whole shot: the model uploaded, material, box homogenisation and box "
                       "material built on the device (fd23_set_model_box), incident generated on the device, "
                       "the run, seismograms"}
    hbm, peak_kind = load_peaks()
    per_step_ms = ms_max / (args.steps * nt)
    ab = alg_bytes(NX, NZ, NPML, 4) + box_alg_bytes(LB_BW, LB_BW, nring, 4)
    achieved = ab / (per_step_ms * 1e-3) / 1e9
    line = {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "psv_4000x2000_5000steps_box32_linesource_c6", "nx": NX, "nz": NZ,
                       "nt": nt, "box": list(box), "ring_cells": nring, "source": [LB_XS, LB_ZS],
                       "mechanism": list(LB_MECH), "alpha": LB_ALPHA, "box_material": list(sv),
                       "kernel": args.kernel,
                       "cells_counted": "grid cells nx*nz per step (the box's residual field is extra work)",
                       "l2": "inputs larger than L2", "parallelism": "replicas x%d" % world},
            "check": {"seismograms_bit_exact_vs_host_generated_incident": check, "max_abs_u": reached},
            "generator": {"ms_per_shot": gen_ms, "frames": nt + 1,
                          "share_of_shot": gen_ms / (ms_max / args.steps)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": None, "peak_source": peak_kind,
                         "scope": "whole step: sweep + box kernels (the generator is in the time)",
                         "alg_bytes_per_launch": ab, "launch_ms": per_step_ms},
            # per step the sweep and the two one-CTA box kernels of a small box;
            # per shot the generator's points, Green's function, convolution
            # and incident kernels (one frame chunk)
            "gpu_launches": args.steps * (nt * 3 + 4),
            "clocks": clocks,
            "e2e": e2e}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_linebox()
    if rank == 0:
        print(json.dumps(line), flush=True)
    s.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


SH_NX, SH_NZ, SH_H, SH_DT, SH_NT, SH_NPML, SH_F0, SH_NSTA = 800, 400, 10.0, 1e-3, 2000, 20, 10.0, 200


def sh_model():
    vs = np.full((SH_NZ, SH_NX), 2000.0)
    rho = np.full((SH_NZ, SH_NX), 2200.0)
    vs[200:] = 3000.0
    rho[200:] = 2500.0
    return vs, rho


def bench_sh(args, F, torch, rank, world, local, dist):
    nt = min(args.nt, SH_NT)
    vs, rho = sh_model()
    # persistent: the whole shot in one cooperative launch (grid barriers
    # between the update phases); fused: the fused sweep in a CUDA graph
    persist = args.kernel == "persist"
    s = F.Solver("sh", SH_NX, SH_NZ, SH_NPML, SH_H, SH_DT, prec=args.prec, pml_dt=SH_DT,
                 pml_v=float(vs.max()) / SH_H, pml_r=1e-11, pml_fc=SH_F0, device=local,
                 kernel="persist" if persist else "fused")
    s.set_model(None, vs, rho)
    src = F.wavelet_ricker(SH_DT, SH_F0)
    s.set_source(F.SRC_FORCE, SH_NX // 2, 20, np.array([1.0, 0.0]), src, nt)
    rx, rz = F.receivers_line(SH_NSTA // 2, 2, 0, 4, 0)
    s.set_receivers(0, rx, rz)
    b = None if persist else F.Batch([s])
    stream = torch.cuda.ExternalStream(s.stream if persist else b.stream, device=local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda:%d" % local)
    # work plan picked by the autotuner (set-up, not timed)
    tune = b.autotune(10) if b is not None and not args.no_tune else []
    plan = b.plan() if tune else None

    def shot():
        s.reset()
        if persist:
            s.run(nt, 1)
        else:
            b.run(nt, 1)

    def sync():
        if persist:
            s.sync()
        else:
            b.sync()

    for _ in range(args.warmup):
        shot()
    sync()
    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
    if dist:
        dist.barrier()
    ms = 0.0
    for _ in range(args.steps):
        flush.zero_()  # L2 flush between timed shots (not timed)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        shot()
        e1.record(stream)
        sync()
        ms += e0.elapsed_time(e1)
    clocks = sampler.stop() if rank == 0 else None
    ms_max = max_over_ranks(ms, dist)
    cells = SH_NX * SH_NZ
    value = cells * nt * args.steps * world / (ms_max * 1e-3)
    e2e = None
    if not args.no_e2e:
        hvs, hrho = (pinned_copy(torch, a) for a in (vs, rho))
        hout = pinned_like(torch, s.seismograms(0))
        times = []
        for _ in range(max(1, min(args.steps, 2))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.set_model(None, hvs, hrho)
            shot()
            out = s.seismograms(0, hout)
            times.append(time.perf_counter() - t0)
        es = {"f32": 4, "f64": 8, "bf16": 2, "f16": 2}[args.prec]
        # vs and rho as doubles (material built on the device)
        up = 2 * cells * 8
        e2e = {"value": cells * nt / statistics.mean(times) * world, "unit": "cell-updates/s",
               "h2d_bytes_per_step": up, "d2h_bytes_per_step": int(out.nbytes)}
    hbm, peak_kind = load_peaks()
    es = {"f32": 4, "f64": 8, "bf16": 2, "f16": 2}[args.prec]
    per_launch_ms = ms_max / (args.steps * nt)
    ab = (3 * 2 + 3) * es * cells + 2 * 2 * (8 if es == 8 else 4) * (2 * SH_NPML * SH_NZ + SH_NPML * SH_NX)
    achieved = ab / (per_launch_ms * 1e-3) / 1e9
    line = {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.prec,
            "data": "synthetic",
            "config": {"workload": "sh_800x400_2000steps_c0", "nx": SH_NX, "nz": SH_NZ, "nt": nt, "plan": plan,
                       "autotune_trials": len(tune),
                       "source": "10 Hz Ricker line force", "traces": SH_NSTA,
                       "kernel": "persistent cooperative launch per shot" if persist else "fused sweep, one-shot batch graph",
                       "l2": "working set (about 10 MB) L2-resident within a shot; L2 flushed between "
                             "timed shots", "parallelism": "replicas x%d" % world},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": None, "peak_source": peak_kind,
                         "note": "L2-resident working set: the HBM fraction is not meaningful here",
                         "alg_bytes_per_launch": ab, "launch_ms": per_launch_ms},
            "gpu_launches": args.steps * (1 if persist else nt + 1), "clocks": clocks, "e2e": e2e}
    if rank == 0 and not args.no_cpu:
        from oracle import fd23_oracle as O
        mat, _, _ = O.sh_material(vs, rho, SH_H, SH_DT)
        bck = O.cpml_sh(SH_NX, SH_NZ, SH_NPML, SH_DT, 1e-11, float(vs.max()) / SH_H, SH_F0)
        terms = O.source_terms("sh", 2, SH_NX, SH_NX // 2, 20, np.array([1.0, 0.0]), SH_H, SH_DT,
                               O.ricker(SH_DT, SH_F0), nt)
        rec = np.asarray(rx) + np.asarray(rz) * SH_NX
        O.sh_run("f32", SH_NX, SH_NZ, SH_NPML, 0, mat, bck, terms, rec, 10)
        t0 = time.perf_counter()
        O.sh_run("f32", SH_NX, SH_NZ, SH_NPML, 0, mat, bck, terms, rec, 400)
        tt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": cells * 400 / tt, "unit": "cell-updates/s", "cores": os.cpu_count() or 1,
                                "kind": "port",
                                "sample": "400 steps of the SH grid (%.1f s), FP32 oracle, all threads" % tt}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if b is not None:
        b.close()
    s.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def batch_shots(seed=7, nshot=NSHOT_B):
    """Seeded shot table of the batched workload: grid, model seed, Ricker
    frequency, source column."""
    rng = np.random.default_rng(seed)
    shots = []
    for k in range(nshot):
        nx = int(rng.integers(1000, 4001))
        nz = int(rng.integers(500, 2001))
        shots.append(dict(nx=nx, nz=nz, mseed=int(rng.integers(1 << 30)), f0=float(rng.uniform(8.0, 25.0)),
                          xs=int(rng.integers(NPML + 20, nx - NPML - 20))))
    return shots


def layered_model(nx, nz, seed):
    """12 seeded flat layers, vp ~ U[1500, 4500] m/s, times 1 + a smooth 5 %
    perturbation (a coarse Gaussian field, bilinear upsampled); vs = vp/1.73,
    rho = 310 vp^0.25."""
    rng = np.random.default_rng(seed)
    bounds = np.sort(rng.choice(np.arange(nz // 20, nz - nz // 20), size=11, replace=False))
    vel = rng.uniform(1500.0, 4500.0, size=12)
    layer = np.searchsorted(bounds, np.arange(nz), side="right")
    cz, cx = max(2, nz // 40), max(2, nx // 40)
    coarse = rng.standard_normal((cz, cx))

    def lin(n, c):  # bilinear upsampling weights, c coarse points to n
        x = np.linspace(0.0, c - 1.0, n)
        i0 = np.minimum(np.floor(x).astype(np.int64), c - 2)
        return i0, x - i0

    iz, wz = lin(nz, cz)
    ix, wx = lin(nx, cx)
    rows = coarse[:, ix] * (1.0 - wx) + coarse[:, ix + 1] * wx
    pert = rows[iz] * (1.0 - wz)[:, None] + rows[iz + 1] * wz[:, None]
    pert *= 0.05 / np.abs(pert).max()
    vp = vel[layer][:, None] * (1.0 + pert)
    return vp, vp / 1.73, 310.0 * vp ** 0.25


def bench_batch(args, F, torch, rank, world, local, dist):
    nt = min(args.nt, NT_B)
    shots = batch_shots(seed=7 + rank)
    prec = args.prec
    models = [layered_model(d["nx"], d["nz"], d["mseed"]) for d in shots]

    def make(d, m, p):
        vp, vs, rho = m
        s = F.Solver("psv", d["nx"], d["nz"], NPML, H, DT, prec=p, pml_dt=DT, pml_v=float(vp.max()) / H,
                     pml_r=1e-11, pml_fc=d["f0"], device=local, kernel="fused")
        s.set_model(vp, vs, rho)
        s.set_source(F.SRC_EXPLOSION, d["xs"], 20, None, F.wavelet_ricker(DT, d["f0"]), nt)
        dx = max(1, (d["nx"] - 2 * NPML) // NSTA_B)
        for f, z in ((0, 0), (1, 1)):
            rx, rz = F.receivers_line(NSTA_B, NPML + 1, z, dx, 0)
            s.set_receivers(f, rx, rz)
        return s

    cells = sum(d["nx"] * d["nz"] for d in shots)
    solvers = [make(d, m, prec) for d, m in zip(shots, models)]
    b = F.Batch(solvers)
    stream = torch.cuda.ExternalStream(b.stream, device=local)
    tune = b.autotune(5)
    plan = b.plan()

    def shot():
        for s in solvers:
            s.reset()
        b.run(nt, 1)

    def sync():
        b.sync()

    for _ in range(args.warmup):
        shot()
    sync()
    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for s in solvers:
        s.reset()
    e0.record(stream)
    for k in range(args.steps):
        if k:
            for s in solvers:
                s.reset()
        b.run(nt, 1)
    e1.record(stream)
    b.sync()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop() if rank == 0 else None
    ms_max = max_over_ranks(ms, dist)
    value = cells * nt * args.steps * world / (ms_max * 1e-3)
    seis = [(s.seismograms(0), s.seismograms(1)) for s in solvers]

    # the same shots one by one with the plain single-shot FP32 solver
    single = None
    if rank == 0 and not args.no_cpu:
        t_single = 0.0
        for d, m in zip(shots, models):
            s = make(d, m, "f32")
            st = torch.cuda.ExternalStream(s.stream, device=local)
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.run(2, 1)
            s.reset()
            s.sync()
            a0.record(st)
            s.run(nt, 1)
            a1.record(st)
            s.sync()
            t_single += a0.elapsed_time(a1)
            s.close()
        single = {"value": cells * nt / (t_single * 1e-3), "unit": "cell-updates/s",
                  "what": "the same 64 shots run one after another with the plain single-shot FP32 solver"}

    # accuracy of 16-bit storage: seismograms against FP64 runs of a subset
    accuracy = None
    if rank == 0 and prec in ("bf16", "f16"):
        pick = np.random.default_rng(11).choice(len(shots), size=NCHECK_B, replace=False)
        errs = []
        for k in pick:
            r = make(shots[k], models[k], "f64")
            r.run(nt, 1)
            ref = np.concatenate([r.seismograms(0).ravel(), r.seismograms(1).ravel()])
            got = np.concatenate([seis[k][0].ravel(), seis[k][1].ravel()]).astype(np.float64)
            errs.append(float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
            r.close()
        accuracy = {"seismogram_rel_l2_vs_fp64": {"max": max(errs), "median": float(np.median(errs)),
                                                  "shots": [int(k) for k in pick], "per_shot": errs}}

    e2e = None
    if not args.no_e2e:
        hmodels = [tuple(pinned_copy(torch, a) for a in m) for m in models]
        hout = [(pinned_like(torch, s.seismograms(0)), pinned_like(torch, s.seismograms(1))) for s in solvers]
        times = []
        for _ in range(max(1, min(args.steps, 2))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for s, m in zip(solvers, hmodels):
                s.set_model(*m)
            shot()
            out = [(s.seismograms(0, hu), s.seismograms(1, hw)) for s, (hu, hw) in zip(solvers, hout)]
            times.append(time.perf_counter() - t0)
        es = {"f32": 4, "f64": 8, "bf16": 2, "f16": 2}[prec]
        e2e = {"value": cells * nt / statistics.mean(times) * world, "unit": "cell-updates/s",
               "h2d_bytes_per_step": 3 * cells * 8,
               "d2h_bytes_per_step": sum(a.nbytes + w.nbytes for a, w in out),
               "note": "per step = one whole batch of shots: material build + upload, the run, seismograms"}
    hbm, peak_kind = load_peaks()
    es = {"f32": 4, "f64": 8, "bf16": 2, "f16": 2}[prec]
    per_launch_ms = ms_max / (args.steps * nt)
    ab = sum(alg_bytes(d["nx"], d["nz"], NPML, es) for d in shots)
    achieved = ab / (per_launch_ms * 1e-3) / 1e9
    line = {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": prec,
            "data": "synthetic",
            "config": {"workload": "psv_batch64_3000steps_c4", "shots": len(shots), "nt": nt,
                       "cells_per_step": cells, "grids": [[d["nx"], d["nz"]] for d in shots],
                       "prec": prec, "plan": plan, "autotune_trials": len(tune),
                       "l2": "inputs larger than L2", "parallelism": "replicas x%d" % world},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": None, "peak_source": peak_kind,
                         "scope": "one batched sweep launch over all shots",
                         "alg_bytes_per_launch": ab, "launch_ms": per_launch_ms},
            "gpu_launches": args.steps * (nt + len(shots)),
            "clocks": clocks,
            "e2e": e2e}
    if single:
        line["single_shot_fp32"] = single
        line["batched_over_single_shot_fp32"] = value / single["value"]
    if accuracy:
        line["accuracy"] = accuracy
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line), flush=True)
    b.close()
    for s in solvers:
        s.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
