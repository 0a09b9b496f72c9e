/*
 * fd23.h -- C ABI of the GB300 (sm_103a) 2-D elastic time-stepping engine.
 *
 * One solver object owns every device buffer of one shot on one GPU.  The
 * calls replace the C++ operator surface of the reference fd23 programs
 * (paths relative to the fd23 project root; PD = PSV/psv_clean_double,
 * PN = PSV/clean_nobox, SH = SH):
 *
 *   reference                                            here
 *   ---------------------------------------------------  ------------------------
 *   PARAM::read_param / make_plan  PD/param/param.cpp:7,160   fd23_create (descriptor)
 *   MATERIAL::get_model            PD/material/material.cpp:101  fd23_set_model
 *   MATERIAL::init_gpu_full        PD/material/cu_material.cu   fd23_set_material
 *   CPML::CPML(PARAM&), CPML(int,CPML&) PD/cpml/cpml.cpp:84,
 *                                  PD/cpml/cu_cpml.cu:5          fd23_create / fd23_set_cpml
 *   gaussian/trapozoid + cu_point_source(_p)
 *                                  PD/source/waveform.cpp:8,27,
 *                                  PD/point_source/cu_point_source.cu:6,66
 *                                                                fd23_set_source / _terms
 *   RECORD::init_line/init_list/cu_init_record
 *                                  PD/record/cu_record.cu:12,30,79  fd23_set_receivers
 *   cu_step_stress/cu_step_velocity + the time loop
 *                                  PD/fd/fd.h:18-19, PN/main.cpp:117-170  fd23_run
 *   RECORD::cu_record/cu_flush     PD/record/cu_record.cu:154,148   fd23_get_seismograms
 *   FIELD::cu_save_state/cu_load_restart, CPML::cu_save_state
 *                                  PN/field/cu_field.cu:26,41;
 *                                  PN/cpml/cu_cpml.cu:92,109     fd23_get_state / fd23_set_state
 *   BOX::init_box                  PD/box/box.cpp:10-119        fd23_set_box, fd23_box_ring_*
 *   MATERIAL::init_for_box_from_full PD/material/material.cpp:39  fd23_box_material
 *                                  (with get_model + init_box on the device:
 *                                                                fd23_set_model_box)
 *   BOX::setboxsource / cu_copy_source
 *                                  PD/box/box.cpp:120, PD/box/cu_box.cu:35
 *                                         fd23_box_incident_from_displacement + fd23_set_box_incident
 *                                         (or fd23_set_box_incident_async)
 *   BOX::cu_addsource/cu_subsource, cu_step_stress_r/_velocity_r
 *                                  PD/box/cu_box.cu:55,71; PD/fd/cu_fd.cu:504,523  fd23_run (box set)
 *   the box-source generator ntde_line (compute_pQpW_mathematica + cu_con)
 *                                  PD/source/source_line.cpp:196-410,
 *                                  PD/source/cu_source.cu:2-42  fd23_line_source_planes,
 *                                                                fd23_set_box_line_source
 *
 * Conventions: every call returns FD23_OK (0) or a negative status and never
 * exits the process; fd23_strerror() names the status.  Host arrays passed in
 * are copied; host output buffers belong to the caller.  Arrays are row-major
 * with x fastest: element (ix, iz) of an nx-by-nz grid is at ix + iz*nx, and
 * iz = 0 is the free surface.  One solver must be driven from one host thread
 * at a time.
 */
#ifndef FD23_H_
#define FD23_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define FD23_OK 0
#define FD23_ERR_ARG (-1)       /* invalid argument or size */
#define FD23_ERR_CUDA (-2)      /* a CUDA runtime call failed */
#define FD23_ERR_UNSTABLE (-3)  /* CFL check failed (stab > 1), PD/material/material.cpp:304 */
#define FD23_ERR_ORDER (-4)     /* call made before what it depends on */
#define FD23_ERR_NOMEM (-5)     /* device allocation failed */
#define FD23_ERR_NONFINITE (-6) /* watchdog found NaN/Inf in the wavefield */
#define FD23_ERR_TIMEOUT (-7)   /* a bounded device-side wait gave up */
#define FD23_ERR_UNSUPPORTED (-8)

/* ---- enums ---- */
enum fd23_wave { FD23_PSV = 0, FD23_SH = 1 };
/* storage/arithmetic forms.  F32 and F64 store and compute in that type;
 * BF16 and F16 store wavefields and material in 16 bits and compute in FP32. */
enum fd23_prec { FD23_F32 = 0, FD23_F64 = 1, FD23_BF16 = 2, FD23_F16 = 3 };
/* kernel choice: AUTO picks the fused single-pass sweep.  PERSIST (an
 * addition for small grids whose fields sit in L2, where a launch per step
 * costs more than the step's work) runs a whole fd23_run in one cooperative
 * launch of the two-pass updates, grid barriers between the phases; results
 * equal TWOPASS bit for bit.  A PERSIST solver with a box steps like TWOPASS;
 * batches take FUSED solvers only.  FUSED2 (P-SV, F32 only; an addition)
 * advances two time steps per launch of a fused sweep that reads and writes
 * every wavefield once per two steps; results equal FUSED bit for bit.  An
 * odd step, and runs with a box, tile windows or a material table, use the
 * one-step sweep. */
enum fd23_kernel {
    FD23_KERNEL_AUTO = 0,
    FD23_KERNEL_FUSED = 1,
    FD23_KERNEL_TWOPASS = 2,
    FD23_KERNEL_PERSIST = 3,
    FD23_KERNEL_FUSED2 = 4
};
/* field ids (source terms, receivers, state) */
enum fd23_psv_field { FD23_U = 0, FD23_W = 1, FD23_TXX = 2, FD23_TXZ = 3, FD23_TZZ = 4 };
enum fd23_sh_field { FD23_V = 0, FD23_TX = 1, FD23_TZ = 2 };
/* point-source kinds (reference stype / srctype) */
enum fd23_source_kind {
    FD23_SRC_EXPLOSION = 1, /* Mxx = Mzz = 1, PN/point_source/cu_point_source.cu:16-20 */
    FD23_SRC_FORCE = 2,     /* SH line force on V, SH/point_source/cu_point_source.cu:162 */
    FD23_SRC_MOMENT = 3,    /* stype 3, PD/point_source/cu_point_source.cu:6-64 */
    FD23_SRC_MOMENT_P = 13  /* stype 13 'p' dipole, running-sum wavelet, :66-146 */
};

typedef struct fd23_solver fd23_solver;

typedef struct {
    int wave;      /* fd23_wave */
    int prec;      /* fd23_prec */
    int nx, nz;    /* grid (any size >= 2*npml+1; no multiple-of-32 rule) */
    int npml;      /* CPML width in cells */
    int topabsorb; /* 0: free surface at iz = 0 (reference default); 1: CPML on top */
    double h, dt;  /* grid spacing and time step (same units as the model) */
    double pml_dt, pml_v, pml_r, pml_fc; /* CPML profile parameters, PD/cpml/cpml.cpp:7 */
    int device;    /* CUDA device ordinal */
    int kernel;    /* fd23_kernel */
} fd23_desc;

/* ---- lifecycle ---- */
int fd23_create(const fd23_desc *desc, fd23_solver **out);
void fd23_destroy(fd23_solver *s);
const char *fd23_strerror(int status);
int fd23_version(void);

/* ---- model / material ----
 * fd23_set_model: vp, vs, den rasters (nx*nz, FP64).  Runs the CFL check,
 * stores *stab, uploads the rasters and builds the staggered, dt/h-scaled
 * material on the device in FP64 with every edge rule of
 * MATERIAL::get_model (PD/material/material.cpp:156-306; SH:
 * SH/material/material.cpp:75-125), in the host builder's operation order
 * (fd23_build_material gives the same values).  The 16-bit forms then scale
 * and round it as fd23_set_material does.  vp is unused for SH and may be
 * NULL.
 * fd23_set_material: already-built arrays, FP64, concatenated
 * (P-SV: LAM, MU, MUA, BU, BW; SH: MUX, MUZ, BV), each nx*nz. */
int fd23_set_model(fd23_solver *s, const double *vp, const double *vs, const double *den,
                   double *stab);
int fd23_set_material(fd23_solver *s, const double *mat);

/* ---- CPML ----
 * fd23_create builds the coefficients from the descriptor.  fd23_set_cpml
 * replaces them: b | c | k blocks, FP64, each block
 * P-SV: Txx_x, Txz_x, U_x, W_x (nx each) then Tzz_z, Txz_z, U_z, W_z (nz each);
 * SH:   Tx_x, V_x (nx each) then Tz_z, V_z (nz each). */
int fd23_set_cpml(fd23_solver *s, const double *bck);

/* ---- source ----
 * fd23_set_source: reference point source.  moment = (Mxx, Mxz, Mzz) for
 * P-SV or (Mxy, Mzy) for SH, unscaled (the 1/(pi*sqrt(2)*h^2) factor is
 * applied here); may be NULL for EXPLOSION.  src = wavelet as s(t)*dt
 * (lsrc samples), nt_max = number of steps the amplitude table covers.
 * fd23_set_source_terms: explicit injections; term t adds
 * amp[t*nt_amp + it] to field[t] at (ix[t], iz[t]) right after the stress
 * update of step it (terms applied in order). */
int fd23_set_source(fd23_solver *s, int kind, int xs, int zs, const double *moment,
                    const double *src, int lsrc, int nt_max);
int fd23_set_source_terms(fd23_solver *s, int nterms, const int *field, const int *ix,
                          const int *iz, const double *amp, int nt_amp);
/* Helpers: wavelets as s(t)*dt (PD/source/waveform.cpp:8-47); return lsrc or
 * a negative status.  ricker is an addition: t0 = 1.2/f0 when t0 <= 0. */
int fd23_wavelet_gaussian(double dt, int alpha, double *out, int cap);
int fd23_wavelet_trapezoid(double dt, double t1, double t2, double t3, double *out, int cap);
int fd23_wavelet_ricker(double dt, double f0, double t0, double *out, int cap);
/* moment tensor projections from strike/dip/rake/azimuth (degrees) */
void fd23_moment_psv(double strike, double dip, double rake, double azimuth, double out3[3]);
void fd23_moment_sh(double strike, double dip, double rake, double azimuth, double out2[2]);

/* ---- receivers ----
 * Positions as given (the reference records each station as the pair
 * (x, z), (x-1, z); fd23_receivers_line builds that list).  field is any
 * wavefield id: the reference records U and W (V for SH); stress receivers
 * are an addition (they record the stress after the step's update). */
int fd23_set_receivers(fd23_solver *s, int field, const int *rx, const int *rz, int n);
int fd23_receivers_line(int nsta, int ix0, int iz0, int idx, int idz, int *rx, int *rz);

/* ---- time stepping ----
 * Advances nsteps steps from the current step counter.  At every step it
 * with it % itrecord == 0 the receivers are sampled after the velocity
 * update.  Asynchronous on the solver's stream; fd23_sync waits. */
int fd23_run(fd23_solver *s, int nsteps, int itrecord);
int fd23_sync(fd23_solver *s);
/* records so far for a receiver field; out holds nrec_steps x n values in the
 * compute type (double for F64, float otherwise); *nrec_steps returns the
 * number of recorded steps. */
int fd23_get_seismograms(fd23_solver *s, int field, void *out, size_t out_bytes,
                         int *nrec_steps);
/* zero wavefields, memory variables, records and the step counter */
int fd23_reset(fd23_solver *s);
/* the cudaStream_t every launch of this solver goes to (for event timing) */
int fd23_get_stream(fd23_solver *s, void **stream);
/* device address of wavefield `field` (storage order, FD23_U ..) in the
 * buffer set the solver currently reads, and its stored element count: the
 * padded layout, nx*nz cells plus zero padding, of the storage type (for the
 * 16-bit forms the stored values carry the solver's power-of-two scales).
 * Valid until the next run; for zero-copy reads such as
 * fd23_sum_squares_noalloc.  No counterpart in the reference (its FIELD
 * members are public device pointers, PD/field/field.h). */
int fd23_get_field_device(fd23_solver *s, int field, void **dev_ptr, size_t *elems);
int fd23_get_step(fd23_solver *s, int *it);

/* ---- state (restart) ----
 * Reference state layout (PN/main.cpp:293-317): P-SV U, W, Txx, Txz, Tzz
 * (nx*nz each) then psi Txx_x, Txz_x, U_x, W_x (2*npml*nz each) then psi
 * Tzz_z, Txz_z, U_z, W_z (2*npml*nx each); SH V, Tx, Tz, psi Tx_x, V_x,
 * Tz_z, V_z.  Element type = compute type.  set_state also sets the step
 * counter to it0 (the reference's nt0). */
size_t fd23_state_bytes(fd23_solver *s);
int fd23_get_state(fd23_solver *s, void *buf, size_t bytes);
int fd23_set_state(fd23_solver *s, const void *buf, size_t bytes, int it0);

/* ---- hybrid box (P-SV, FD23_F32 / FD23_F64) ----
 * A box is the grid cells [x0, x0+bx) x [z0, z0+bz), bx, bz >= 16 (the
 * reference's box is bw x bw around the source at x0 = xs + (bw+1)/2 + 1 - bw,
 * likewise z0; PD/box/box.cpp:26-45).  It holds a residual field r with its
 * own material.  Two 4-cell rings couple r and the grid field g through an
 * incident field s given on the ring cells every step:
 *   sub ring (the outer 4 cells of the box):    r = g - s
 *   add ring (the next 4 cells inward):         g = r + s
 * around both half-steps, in the order of PD/main.cpp:153-199; r advances
 * on box cells 4 .. n-5 with 8th-order stencils, no CPML (PD/fd/fd.cpp:63,208).
 * fd23_set_box: bmat = box material LAM, MU, MUA, BU, BW (dt/h scaled,
 *   bx*bz each, FP64) or NULL for the cut of the solver's material; r starts
 *   at zero.  bx = bz = 0 removes the box.  FD23_ERR_UNSUPPORTED for SH and
 *   the 16-bit forms.
 * fd23_set_box_incident: incident field of steps it0 .. it0+nsteps-1, laid out
 *   [step][U W Txx Txz Tzz][nring] in the compute type; ring order = sub
 *   ring then add ring, each row by row (fd23_box_ring_cells).  U, W are the
 *   velocities before the step, the stresses those after its stress update.
 *   Copied to the device before the call returns.  fd23_run fails with
 *   FD23_ERR_ORDER for a step it does not cover.
 * fd23_get_box_state / fd23_set_box_state: r as U W Txx Txz Tzz, bx*bz each,
 *   compute type (fd23_box_state_bytes).
 * A box excludes tile step windows (fd23_set_punch) and material tables
 *   (fd23_set_material_table): FD23_ERR_UNSUPPORTED. */
int fd23_set_box(fd23_solver *s, int x0, int z0, int bx, int bz, const double *bmat);
/* fd23_set_model and the reference's box set-up in one call, on the device:
 * the material from vp, vs, den (fd23_set_model), then the box at (x0, z0)
 * homogenised towards the source material src_vp, src_vs, src_den and its
 * box material installed, as fd23_box_material + fd23_set_material +
 * fd23_set_box(..., bmat) do on the host (MATERIAL::init_for_box_from_full,
 * PD/material/material.cpp:39-97), with the same values.  replaced (may be
 * NULL) receives the number of box cells that took the source material, bmat
 * (may be NULL) the box material as fd23_box_material returns it (FP64,
 * 5 x bz x bx: what fd23_set_box_line_source takes). */
int fd23_set_model_box(fd23_solver *s, const double *vp, const double *vs, const double *den, int x0, int z0,
                       int bx, int bz, double src_vp, double src_vs, double src_den, double *stab, int *replaced,
                       double *bmat);
int fd23_set_box_incident(fd23_solver *s, const void *inc, int it0, int nsteps);
/* The same upload without waiting for it: the copy runs on a copy stream in
 * chunks of steps, each box step of the solver waits only for the chunk that
 * holds its incident field, so the upload overlaps the run.  inc must stay
 * valid and unchanged until the solver's work has finished (fd23_sync);
 * page-locked host memory lets the copy run asynchronously. */
int fd23_set_box_incident_async(fd23_solver *s, const void *inc, int it0, int nsteps);
size_t fd23_box_state_bytes(fd23_solver *s);
int fd23_get_box_state(fd23_solver *s, void *buf, size_t bytes);
int fd23_set_box_state(fd23_solver *s, const void *buf, size_t bytes);
/* Ring geometry (host only): sizes (returns nsub + nadd), the ring position of
 * box cell (bi, bj) (-1 if in neither ring), and the grid cells of every ring
 * position (ix, iz: nsub + nadd entries each; returns that count). */
int fd23_box_ring_size(int bx, int bz, int *nsub, int *nadd);
int fd23_box_ring_index(int bx, int bz, int bi, int bj);
int fd23_box_ring_cells(int x0, int z0, int bx, int bz, int *ix, int *iz);
/* BOX::setboxsource (host only, FP64): the incident field of one step on the
 * ring cells (out: 5 x nring) from the displacement planes of this step
 * (u_old, w_old) and the next (u_new, w_new), each (bx+8) x (bz+8), box cell
 * (i, j) at plane (i+4, j+4); bmat as for fd23_set_box (LAM, MU, MUA used).
 * Returns nring. */
int fd23_box_incident_from_displacement(int bx, int bz, double dt, const double *bmat,
                                        const double *u_old, const double *w_old,
                                        const double *u_new, const double *w_new, double *out);
/* MATERIAL::init_for_box_from_full (host only, FP64): box material from the
 * grid material mat (LAM MU MUA BU BW, nx*nz each); box cells that differ
 * from the homogeneous source material (src_vp, src_vs, src_den) by more
 * than 1e-4 are set to it in mat too.  Returns the number of such cells. */
int fd23_box_material(int nx, int nz, double *mat, int x0, int z0, int bx, int bz, double src_vp,
                      double src_vs, double src_den, double dt, double h, double *bmat);

/* ---- box-source generator (the reference's ntde_line program,
 * PD/source/source_line.cpp:307-410) ----
 * Displacement planes of a line moment source in a homogeneous full space,
 * the incident field of the hybrid box.  Plane cell (p, q), p < px, q < pz,
 * is ox + p, oz + q cells from the source cell; the U plane samples the
 * point ((ox+p) + 0.5 - sx, (oz+q) - sz) * h, the W plane
 * ((ox+p) - sx, (oz+q) - 0.5 - sz) * h (x right, z down).  Each sample is
 * the time derivative of the closed-form 2-D Green's function
 * (compute_pQpW_mathematica, :196-305; FP64), convolved with the wavelet
 * src (s(t) dt values, as fd23_set_source takes) in the reference kernel's
 * order (cu_con, PD/source/cu_source.cu:2-42).  Samples before a point's
 * P arrival are zero; points within one step's travel of the source give
 * NaN at t = 0 (0/0), as in the reference, and so NaN in the first
 * frames after the convolution.
 * The reference writes frames 0 .. nt-1 of the square box around its
 * source: px = pz = bw + 8, ox = oz = fd23_line_plane_origin(bw),
 * sx = 0.25, sz = -0.25, a = fd23_line_source_coefs(strike, dip, rake,
 * azimuth) (:320-326, theta = azimuth - strike). */
typedef struct {
    int px, pz;          /* plane size in cells */
    int ox, oz;          /* source-relative cell offset of plane cell (0, 0) */
    double h, dt;
    double vp, vs, den;  /* the homogeneous medium (srcpvel, srcsvel, srcden) */
    double a[3];         /* radiation coefficients A1, A2, A3 */
    double sx, sz;       /* source point inside its cell, in cells */
} fd23_line_desc;
int fd23_line_source_coefs(double strike, double dip, double rake, double azimuth, double a[3]);
int fd23_line_plane_origin(int bw);
/* Frames it0 .. it0+nframes-1 computed on the GPU `device`, written to the
 * host buffer out as [frame][U plane, W plane][pz][px] doubles (the layout
 * of the reference's source file).  FD23_ERR_ARG for sizes <= 0, lsrc < 1
 * or lsrc > 8192, a non-positive h, dt, vp, vs or den. */
int fd23_line_source_planes(int device, const fd23_line_desc *d, const double *src, int lsrc, int it0,
                            int nframes, double *out);
/* The box's incident field of steps it0 .. it0+nsteps-1 generated on the
 * device from the line source: frames it0 .. it0+nsteps of the planes the
 * ring stencils read (px = bx+8, pz = bz+8, plane cell (i+4, j+4) = box
 * cell (i, j)) followed by the setboxsource step with the box material
 * bmat (FP64, as for fd23_set_box; LAM, MU, MUA used), in place of a
 * fd23_set_box_incident upload.  Same values as
 * fd23_line_source_planes -> fd23_box_incident_from_displacement ->
 * fd23_set_box_incident.  FD23_ERR_ORDER without a box, FD23_ERR_ARG for
 * planes of another size. */
int fd23_set_box_line_source(fd23_solver *s, const fd23_line_desc *d, const double *src, int lsrc,
                             const double *bmat, int it0, int nsteps);

/* ---- batched shots (no counterpart in the reference, which runs one shot
 * per process, PD/main.cpp:43-183) ----
 * A batch advances several solvers -- shots of any grid sizes, one wave type,
 * one precision, one device, fused sweep, no box -- in lockstep: every time
 * step is one launch of the sweep over all shots.  The solvers keep their
 * buffers, sources and receivers; after fd23_batch_run their step counters,
 * states and seismograms are as if each had run alone (bit for bit).  All
 * solvers must be at the same step with the same record count.  The launches
 * of a run are captured into a CUDA graph; a later run over the same step
 * range (e.g. after fd23_reset of every solver) replays it.  Work is queued on
 * the batch's stream, ordered after and before the solvers' own streams.
 * fd23_batch_set_graph(b, 0) launches step by step instead. */
typedef struct fd23_batch fd23_batch;
int fd23_batch_create(fd23_solver *const *solvers, int n, fd23_batch **out);
void fd23_batch_destroy(fd23_batch *b);
int fd23_batch_run(fd23_batch *b, int nsteps, int itrecord);
int fd23_batch_sync(fd23_batch *b);
int fd23_batch_get_stream(fd23_batch *b, void **stream);
int fd23_batch_set_graph(fd23_batch *b, int on);

/* ---- work-plan autotuner (no counterpart in the reference) ----
 * The fused sweep's work plan: 4-row blocks of 120-column strips, weighted by
 * an estimated cost (wx for blocks touching the x-CPML, wz for the z-CPML and
 * edge rows, 1 otherwise), cut into equal-cost contiguous ranges for
 * per_sm x SMs x oversub CTAs (bands = 0), or strip by strip (bands = 1).
 * fd23_autotune / fd23_batch_autotune time every candidate plan (144: wx
 * 2..7, wz 2..5, oversub 1..3, bands 0..1) for trial_steps steps on the live
 * shot(s), then the five fastest and the 8 half-step
 * neighbours of the best weights for 3 x trial_steps (a single FP32 shot
 * without windows, table or box: then the best plan with fast_iter = 1),
 * restore the wavefields, memory
 * variables and step counters after each trial, and keep the fastest plan
 * of the long trials.  table (cap
 * entries) receives every trial, the second round last; returns the number
 * of trials or a negative status. */
typedef struct {
    double wx, wz;      /* block cost weights */
    int per_sm;         /* resident CTAs per SM */
    int bands;          /* 0: ranges cut strip after strip; 1: every strip cut
                         * on its own, at the same rows as the strips of the
                         * same cost (single-shot plans of one wave or more
                         * CTAs than strips; others fall back to 0) */
    double oversub;     /* CTAs launched per resident slot */
    double ms_per_step; /* measured (0 for the current plan) */
    int fast_iter;      /* 1: the single-shot FP32 sweep with uniform fast
                         * iterations (interior rows of all-interior warps
                         * without per-lane branches; same results), 0: the
                         * plain one.  16-bit storage always takes them; FP64,
                         * the batch and the window / table sweeps ignore it. */
} fd23_tune_entry;
int fd23_autotune(fd23_solver *s, int trial_steps, fd23_tune_entry *table, int cap);
int fd23_batch_autotune(fd23_batch *b, int trial_steps, fd23_tune_entry *table, int cap);
int fd23_batch_get_plan(fd23_batch *b, fd23_tune_entry *current, int *nblocks);
/* fd23_batch_set_plan installs a plan for the batch without timing it (the
 * arguments of fd23_set_plan). */
int fd23_batch_set_plan(fd23_batch *b, const fd23_tune_entry *tune);
/* fd23_set_plan installs a plan without timing it (ms_per_step ignored;
 * per_sm is capped at the residency the device reports; oversub in
 * [1/16, 64]: below 1, part of a wave of CTAs, for small grids);
 * fd23_get_plan reports the current one and its CTA count. */
int fd23_set_plan(fd23_solver *s, const fd23_tune_entry *tune);
int fd23_get_plan(fd23_solver *s, fd23_tune_entry *current, int *nblocks);
/* The work plan for nshots grids under the given parameters (host only, for
 * inspection and tests): items receives 4 ints per item (shot, x0, z0, z1:
 * 120 columns from x0, rows [z0, z1)), off[c] .. off[c+1] indexes the items of
 * CTA c (off needs cap_ctas + 1 entries).  Returns the CTA count.  A shot's
 * strips start at a column xoff, a multiple of 8 in (-120, 0], chosen so that
 * the x-CPML zones fall into the fewest strips (x0 = xoff + 120 k; columns
 * left of 0 are outside the grid). */
int fd23_work_plan(int nshots, const int *nx, const int *nz, const int *npml, const int *topabsorb,
                   int sms, const fd23_tune_entry *tune, int *items, int cap_items, int *off,
                   int cap_ctas);
/* The same over the live 4-row blocks only (the phase plans of the sweep
 * with tile step windows): live holds, shot after shot, one byte per block
 * (strip-major: strip * ceil(nz/4) + block, 120-column strips from column 0);
 * a shot with no live block gets no CTA. */
int fd23_work_plan_live(int nshots, const int *nx, const int *nz, const int *npml, const int *topabsorb,
                        int sms, const fd23_tune_entry *tune, const unsigned char *live, int *items,
                        int cap_items, int *off, int cap_ctas);

/* ---- diagnostics ----
 * FP64 energy-norm watchdog over the wavefield: sum of squares of all
 * fields in FP64; returns FD23_ERR_NONFINITE when any value is NaN/Inf. */
int fd23_field_norm2(fd23_solver *s, double *norm2);

/* ---- failure-path check ----
 * Runs, on the solver's stream, the sweep's bounded device-side wait on a
 * barrier that nothing completes.  The wait gives up after about 2 s and
 * raises the solver's error flag, exactly as a sweep whose copies never
 * arrive would: fd23_sync then returns FD23_ERR_TIMEOUT, later sweeps
 * return at once, and fd23_reset clears the flag.  For tests of the failure
 * handling; it faults nothing and leaves the GPU usable. */
int fd23_debug_expire_wait(fd23_solver *s);
/* The same check for a FD23_KERNEL_PERSIST solver: one step of its
 * cooperative launch whose first grid barrier waits for one block more than
 * the launch has.  Every block's bounded wait gives up after about 10 ms and
 * raises the error flag: fd23_sync returns FD23_ERR_TIMEOUT, later runs
 * return at once, and fd23_reset clears the flag (the stress update of that
 * step has run, so the wavefields need the reset too).  FD23_ERR_ORDER for
 * other solvers or before the material. */
int fd23_debug_persist_barrier(fd23_solver *s);

/* ---- allocation-free watchdog ----
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory (programs whose device memory belongs to another allocator: a
 * framework's caching allocator, a pool sized at start-up): sums the squares
 * of nfields caller-owned device arrays of n elements each (element type
 * prec) in FP64 into *sum and sets *nonfinite when any value is NaN or Inf
 * -- the same quantity fd23_field_norm2 computes for a solver -- without
 * allocating.  Its partial sums live in a fixed 16 KiB file-scope device
 * array that every GPU loading the library keeps until exit.  At most 8
 * arrays per call (more returns FD23_ERR_ARG); every array must be device
 * memory of the current device and `stream` (a cudaStream_t, NULL = default)
 * must belong to it (FD23_ERR_ARG otherwise).  The call waits for its stream,
 * so it cannot run on a stream that is being captured: there it returns
 * FD23_ERR_UNSUPPORTED without touching the stream.  All calls share the
 * scratch array, so calls that overlap on the GPU race; serialize them. */
int fd23_sum_squares_noalloc(int prec, const void *const *fields, int nfields, size_t n,
                             void *stream, double *sum, int *nonfinite);

/* ---- material table (mktable) ----
 * Replaces MATERIAL::mktable (PD/material/mktable.cpp:43-106; called by
 * SH/main.cpp:154) and the usetable reads of the sweep kernels
 * (PD/fd/cu_fd.cu:262-270, SH/fd/cu_fd.cu:117,219).  on = 1 turns the
 * solver's material into one index byte per cell and a table of the distinct
 * material tuples (storage values, matched bit for bit, so results are
 * identical); the sweeps then read one byte per cell instead of 5 (P-SV) or
 * 3 (SH) material values.  Returns the number of table entries (the zero
 * tuple of the padding included), FD23_ERR_UNSUPPORTED past 256 entries or
 * with a hybrid box, FD23_ERR_ORDER before the material.  While on, every
 * fd23_set_material / fd23_set_model rebuilds the table; one that no longer
 * fits turns the table off.  on = 0 removes it.  Batches need tables in all
 * shots or in none. */
int fd23_set_material_table(fd23_solver *s, int on);

/* ---- usepunch: tile step windows ----
 * Replaces the SLIDE object (PD/slide/slide.h:4-13, PD/slide/cu_slide.cu:6-66)
 * and its test in the sweep kernels (PD/fd/cu_fd.cu:16-23, called at :249
 * and :404; SH/fd/cu_fd.cu:106,206).  The grid is cut into tiles of 32
 * columns x 16 rows, nbx = ceil(nx/32) by nbz = ceil(nz/16)
 * (fd23_punch_tiles); the reference requires whole tiles.  The cells of
 * tile (ix/32, iz/16) are updated at step it (0-based, counted across
 * restarts as PN/main.cpp:115-117) only while first < it < last; otherwise
 * their stresses, velocities and memory variables keep their values.  Point
 * sources and receivers act as without windows.
 * fd23_punch_windows: first = int((tmin - before)/dt), last = int((tmax +
 *   after)/dt) per tile from travel times t[nz][nx] (tmin, tmax over the
 *   tile); elem_bytes 8 = double times and arithmetic (PD), 4 = float (PN,
 *   SH).  The conversion to int saturates; NaN gives 0.
 * fd23_read_punch: the same from a raw travel-time file (the reference's
 *   `timefile`, nx*nz values of elem_bytes each).
 * fd23_set_punch: installs windows [nbz][nbx] (first, last); both NULL
 *   removes them.  Works with both sweeps and in batches;
 *   FD23_ERR_UNSUPPORTED with a hybrid box.  The fused sweep skips tiles
 *   left alone at this step and the last (and without a live source term). */
int fd23_punch_tiles(int nx, int nz, int *nbx, int *nbz);
int fd23_punch_windows(const void *times, int elem_bytes, int nx, int nz, double before, double after,
                       double dt, int *first, int *last);
int fd23_read_punch(const char *timefile, int elem_bytes, int nx, int nz, double before, double after, double dt,
                    int *first, int *last);
int fd23_set_punch(fd23_solver *s, const int *first, const int *last, int nbx, int nbz);
/* With windows the fused sweep of a single solver plans its work per phase
 * of `steps` steps (default 128) over the 4-row blocks live in that phase, so
 * every step's work spreads over the whole GPU; 0 keeps the one plan of the
 * whole grid (batches always do). */
int fd23_set_punch_phase(fd23_solver *s, int steps);

/* ---- model and station input (host only) ----
 * fd23_read_model: a ".mdl" polygon model (BACK / POLY / DEF commands,
 * PD/model/model.cpp:240-369, rasterised at (ix*h, iz*h) as get_elas_model,
 * :175-232) or raster files <name>.vp, .vs, .den (float32 nx*nz,
 * PD/model/util.cpp:12-22), into FP64 arrays of nx*nz.
 * fd23_read_stations: a station file of "z x" lines (PD/record/cu_record.cu:
 * 30-76), each station listed as the pair (x, z), (x-1, z); returns the
 * number of receivers (2 per station); cap = 0 only counts. */
int fd23_read_model(const char *name, int nx, int nz, double h, double *vp, double *vs, double *den);
int fd23_read_stations(const char *path, int *rx, int *rz, int cap);

/* ---- host-only builders (no GPU needed) ----
 * The same FP64 set-up fd23_set_model / fd23_create / fd23_set_source use,
 * exposed for callers that build inputs themselves.
 * fd23_build_material: out = nmat*nx*nz (see fd23_set_material); returns
 *   FD23_OK or FD23_ERR_UNSTABLE (out is filled either way).
 * fd23_build_cpml: returns the element count written (3 * block size).
 * fd23_build_source_terms: returns the number of terms (amp: terms x nt). */
int fd23_build_material(int wave, int nx, int nz, double h, double dt, const double *vp,
                        const double *vs, const double *den, double *out, double *stab);
int fd23_build_cpml(int wave, int nx, int nz, int npml, double pml_dt, double pml_r, double pml_v,
                    double pml_fc, double *out, size_t out_elems);
int fd23_build_source_terms(int wave, int kind, int xs, int zs, const double *moment, double h,
                            double dt, const double *src, int lsrc, int nt, int *field, int *ix,
                            int *iz, double *amp, int max_terms);

#ifdef __cplusplus
}
#endif
#endif /* FD23_H_ */
