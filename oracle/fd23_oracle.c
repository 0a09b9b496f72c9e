/*
 * fd23 CPU oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is a plain-C restatement of the reference fd23 algorithms for the
 * 2-D elastic time-stepping hot path.  It exists so that tests, the smoke check
 * and the CPU-baseline leg of the benchmark can check the CUDA product against
 * an independent implementation.  Nothing in the product library links,
 * loads or calls this code.
 *
 * Parity pins (checked by tests/test_oracle_golden.py):
 *   - PSV/t/clean_nobox/TEST/output_U, output_W  (FP32 P-SV, 1024x1024, 2000 steps)
 *   - PSV/psv_clean_double/test/0_U, 0_W         (FP64 P-SV, fluid layer, 2048x1024, 2001 steps)
 *   - PSV/clean_nobox/TEST/tt/state000499 -> state000999 restart pair
 *
 * Arithmetic order.  Every derivative and every update is written with an
 * explicit operation sequence (products, differences and fused multiply-adds
 * named one by one).  The CUDA kernels of the product follow the same
 * sequence, so in FP64 and FP32 the oracle and the GPU agree bit for bit on
 * the same inputs.  Build with -ffp-contract=off so the compiler adds no
 * fusion of its own.
 *
 * Reference files cited below are relative to the fd23 project root:
 *   PD = PSV/psv_clean_double, PN = PSV/clean_nobox, SH = SH.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* 8th-order staggered coefficient table, rows = stencil order 0..4.
 * PD/param/const.h:1-19 (g_coef). Row 0 and 1 are both the 2nd-order pair. */
static const double OR_COEF[5][4] = {
    {1.0, 0.0, 0.0, 0.0},
    {1.0, 0.0, 0.0, 0.0},
    {9. / 8., 1. / 24., 0.0, 0.0},
    {75. / 64., 25. / 384., 3. / 640., 0.0},
    {1225. / 1024., 245. / 3072., 49. / 5120., 5. / 7168.}};

#define OR_PI 3.14159265358979 /* PD/param/const.h:26 */

/* ------------------------------------------------------------------------- */
/* Material builders (FP64), PD/material/material.cpp:156-282 and            */
/* SH/material/material.cpp:75-105.                                           */
/* ------------------------------------------------------------------------- */

/* P-SV: out = LAM, MU, MUA, BU, BW (each nx*nz, row-major idx = ix + iz*nx),
 * all scaled by dt/h.  Returns 0, or -1 when the reference CFL check
 * (material.cpp:296-306) fails; stab is returned through *stab_out. */
int or_psv_material(int nx, int nz, double h, double dt, const double *vp, const double *vs,
                    const double *den, double *out, double *stab_out)
{
    const long n = (long)nx * nz;
    double *LAM = out, *MU = out + n, *MUA = out + 2 * n, *BU = out + 3 * n, *BW = out + 4 * n;
    for (long k = 0; k < 5 * n; k++) out[k] = 0.0;
    /* material.cpp:156-164 */
    for (long k = 0; k < n; k++) {
        double mu = vs[k] * vs[k] * den[k];
        double lam = vp[k] * vp[k] * den[k] - 2.0 * mu;
        LAM[k] = lam;
        MU[k] = mu;
    }
    /* water-edge stabilisation within 5 cells of left/right/bottom edges,
     * material.cpp:166-201 */
    const int wst = 5;
    for (int iz = 0; iz < nz; iz++) {
        for (int ix = 0; ix < wst && ix < nx; ix++) {
            long k = (long)iz * nx + ix;
            if (vs[k] / vp[k] < 0.01) {
                double mu = vp[k] * vp[k] / 3.0 * den[k];
                LAM[k] = vp[k] * vp[k] * den[k] - 2.0 * mu;
                MU[k] = mu;
            }
        }
        for (int ix = nx - wst; ix < nx; ix++) {
            if (ix < 0) continue;
            long k = (long)iz * nx + ix;
            if (vs[k] / vp[k] < 0.01) {
                double mu = vp[k] * vp[k] / 3.0 * den[k];
                LAM[k] = vp[k] * vp[k] * den[k] - 2.0 * mu;
                MU[k] = mu;
            }
        }
    }
    for (int iz = nz - wst; iz < nz; iz++) {
        if (iz < 0) continue;
        for (int ix = 0; ix < nx; ix++) {
            long k = (long)iz * nx + ix;
            if (vs[k] / vp[k] < 0.01) {
                double mu = vp[k] * vp[k] / 3.0 * den[k];
                LAM[k] = vp[k] * vp[k] * den[k] - 2.0 * mu;
                MU[k] = mu;
            }
        }
    }
    /* buoyancy and harmonic shear averages for rows >= 1, material.cpp:204-233.
     * Quirks kept: BU's right neighbour wraps to the next row (k+1), BW of the
     * last row uses den[k] twice (the guard tests k+nx but reads k-nx), and
     * the MUA denominator holds the m2*m3*m4 term twice. */
    for (int iz = 1; iz < nz; iz++) {
        for (int ix = 0; ix < nx; ix++) {
            long k = (long)iz * nx + ix;
            BU[k] = (k + 1 < n) ? 2.0 / (den[k] + den[k + 1]) : 2.0 / (den[k] + den[k]);
            BW[k] = (k + nx < n) ? 2.0 / (den[k] + den[k - nx]) : 2.0 / (den[k] + den[k]);
            if (ix + 1 < nx && iz + 1 < nz) {
                double m1 = MU[k], m2 = MU[k + 1], m3 = MU[k - nx], m4 = MU[k + 1 - nx];
                double den4 = m2 * m3 * m4 + m1 * m3 * m4 + m1 * m2 * m4 + m2 * m3 * m4;
                if (den4 < 1e-10) den4 = 1e-10;
                MUA[k] = 4.0 * m1 * m2 * m3 * m4 / den4;
            } else {
                MUA[k] = MU[k];
            }
        }
    }
    /* free-surface row edits (Mittet 2002), material.cpp:260-273 */
    for (int ix = 1; ix < nx - 1; ix++) {
        BU[ix] = (ix + 1 < nx) ? 4.0 / (den[ix] + den[ix + 1]) : 4.0 / (den[ix] + den[ix]);
        LAM[ix] = 0.0;
        MU[ix] = 0.5 * MU[ix];
    }
    /* scale by dt/h, material.cpp:275-282 */
    const double fac = dt / h;
    for (long k = 0; k < 5 * n; k++) out[k] *= fac;
    /* stability check, material.cpp:285-306 */
    double vpmax = -99999.0;
    for (long k = 0; k < n; k++)
        if (vp[k] > vpmax) vpmax = vp[k];
    double coefsum = OR_COEF[4][0] + OR_COEF[4][1] + OR_COEF[4][2] + OR_COEF[4][3];
    double stab = vpmax * dt * coefsum * sqrt(2.0) / h;
    if (stab_out) *stab_out = stab;
    return stab > 1.0 ? -1 : 0;
}

/* SH: out = MUX, MUZ, BV (each nx*nz), scaled by dt/h.
 * SH/material/material.cpp:75-105; CFL check on vs :108-125. */
int or_sh_material(int nx, int nz, double h, double dt, const double *vs, const double *den,
                   double *out, double *stab_out)
{
    const long n = (long)nx * nz;
    double *MUX = out, *MUZ = out + n, *BV = out + 2 * n;
    for (int iz = 0; iz < nz; iz++) {
        for (int ix = 0; ix < nx; ix++) {
            long k = (long)iz * nx + ix;
            BV[k] = 1.0 / den[k];
            double m1 = vs[k] * vs[k] * den[k];
            double m2 = (k + 1 < n) ? vs[k + 1] * vs[k + 1] * den[k + 1] : m1;
            double s = m1 + m2;
            if (s < 1e-10) s = 1e-10;
            MUX[k] = 2.0 * m1 * m2 / s;
            m2 = (k - nx >= 0) ? vs[k - nx] * vs[k - nx] * den[k - nx] : m1;
            s = m1 + m2;
            if (s < 1e-10) s = 1e-10;
            MUZ[k] = 2.0 * m1 * m2 / s;
        }
    }
    const double fac = dt / h;
    for (long k = 0; k < 3 * n; k++) out[k] *= fac;
    double vsmax = -99999.0;
    for (long k = 0; k < n; k++)
        if (vs[k] > vsmax) vsmax = vs[k];
    double coefsum = OR_COEF[4][0] + OR_COEF[4][1] + OR_COEF[4][2] + OR_COEF[4][3];
    double stab = vsmax * dt * coefsum * sqrt(2.0) / h;
    if (stab_out) *stab_out = stab;
    return stab > 1.0 ? -1 : 0;
}

/* ------------------------------------------------------------------------- */
/* CPML profile, PD/cpml/cpml.cpp:7-83.                                      */
/* ------------------------------------------------------------------------- */
void or_cpml_profile(int npml, double startpos, int n, double pml_dt, double R, double v,
                     double fc, double *b, double *c, double *k)
{
    const double pml_pos = npml - 0.5;
    const double sigmax = -(2.0 + 1.0) / (2.0 * floor(pml_pos)) * v * log(R);
    const double alphamax = 3.141592653589 * fc;
    const double kmax = 2.0;
    double *d = (double *)calloc((size_t)n, sizeof(double));
    for (int i = 0; i < npml + 2 && i < n; i++) {
        double t = (pml_pos - (i + startpos)) / floor((double)npml);
        if (t > 0) d[i] = t;
    }
    for (int i = n - npml - 2; i < n; i++) {
        if (i < 0) continue;
        double t = ((i + startpos) - (n - 1 - pml_pos)) / floor((double)npml);
        if (t > 0) d[i] = t;
    }
    for (int i = 0; i < n; i++) {
        double sg = sigmax * pow(d[i], 2.0);
        double kp = 1.0 + (kmax - 1.0) * pow(d[i], 2.0);
        double al = alphamax * (1.0 - pow(d[i], 1.0));
        double bb = exp(-(sg / kp + al) * pml_dt);
        double cc = (sg + kp * al < 1e-15) ? 0.0 : sg * (bb - 1.0) / (sg + kp * al) / kp;
        b[i] = bb;
        c[i] = cc;
        k[i] = 1.0 / kp;
    }
    /* frozen edge cells, cpml.cpp:55-64 */
    for (int i = 0; i < 4 && i < n; i++) b[i] = c[i] = k[i] = 0.0;
    for (int i = n - 5; i < n; i++)
        if (i >= 0) b[i] = c[i] = k[i] = 0.0;
    free(d);
}

/* ------------------------------------------------------------------------- */
/* Source-time functions (FP64), PD/source/waveform.cpp:8-47.  Values are     */
/* s(t)*dt.  Return lsrc, or -1 when cap is too small.                       */
/* ------------------------------------------------------------------------- */
int or_gaussian(double dt, int alpha, double *src, int cap)
{
    (void)dt;
    int aint = abs((int)(alpha * 3.0));
    int lsrc = 2 * aint + 1;
    if (lsrc > cap) return -1;
    if (alpha >= 0) {
        for (int i = -aint; i <= aint; i++)
            src[i + aint] = (double)i * exp((double)(-i) * (double)i / ((double)alpha * alpha));
    } else {
        double sum = 0.0;
        for (int i = -aint; i <= aint; i++) {
            src[i + aint] = exp((double)(-i) * (double)i / ((double)alpha * alpha));
            sum += src[i + aint];
        }
        for (int i = 0; i < lsrc; i++) src[i] /= sum;
    }
    return lsrc;
}

int or_trapezoid(double dt, double trap1, double trap2, double trap3, double *src, int cap)
{
    int t1 = (int)(trap1 / dt), t2 = (int)(trap2 / dt), t3 = (int)(trap3 / dt);
    t2 += t1;
    int lsrc = t2 + t3;
    if (lsrc > cap) return -1;
    double amp = (trap2 + 0.5 * (trap1 + trap3)) / dt;
    int p = 0, i;
    for (i = 0; i < t1; i++) src[p++] = i / (t1 * amp);
    for (; i < t2; i++) src[p++] = 1.0 / amp;
    for (i = t3; i > 0; i--) src[p++] = i / (t3 * amp);
    return lsrc;
}

/* Moment tensor projections, PD/point_source/cu_point_source.cu:16-26 (P-SV)
 * and SH/point_source/cu_point_source.cu:16-24 (SH: m[0]=Mxy, m[1]=Mzy). */
void or_moment_psv(double strike, double dip, double rake, double azimuth, double *m3)
{
    double delta = dip * OR_PI / 180.0, lambda = rake * OR_PI / 180.0;
    double phi = (strike - azimuth) * OR_PI / 180.0;
    m3[0] = -(sin(delta) * cos(lambda) * sin(2.0 * phi) +
              sin(2.0 * delta) * sin(lambda) * sin(phi) * sin(phi));
    m3[1] = -(cos(delta) * cos(lambda) * cos(phi) + cos(2.0 * delta) * sin(lambda) * sin(phi));
    m3[2] = sin(2.0 * delta) * sin(lambda);
}

void or_moment_sh(double strike, double dip, double rake, double azimuth, double *m2)
{
    double delta = dip * OR_PI / 180.0, lambda = rake * OR_PI / 180.0;
    double phi = (strike - azimuth) * OR_PI / 180.0;
    m2[0] = sin(delta) * cos(lambda) * cos(2.0 * phi) +
            0.5 * sin(2.0 * delta) * sin(lambda) * sin(2.0 * phi);
    m2[1] = -(cos(delta) * cos(lambda) * sin(phi) - cos(2.0 * delta) * sin(lambda) * cos(phi));
}

/* Field ids used by source terms and state buffers. */
enum { OR_U = 0, OR_W = 1, OR_TXX = 2, OR_TXZ = 3, OR_TZZ = 4 };      /* P-SV */
enum { OR_V = 0, OR_TX = 1, OR_TZ = 2 };                               /* SH   */

/* Point-source injection terms.  Each term adds amp[term*nt + it] to one
 * cell of one field right after the stress update of step it (terms applied
 * in list order, one rounding each).
 *   kind 3  : moment tensor, PD/point_source/cu_point_source.cu:6-64
 *   kind 13 : 'p' dipole with running-sum wavelet and clamp, :66-146
 *   kind 1  : explosion Mxx=Mzz=1, PN/point_source/cu_point_source.cu:16-20
 * m3 = (Mxx, Mxz, Mzz).  src holds s(t)*dt (length lsrc).
 * Returns the number of terms (<= 12). */
int or_psv_source_terms(int kind, int nx, int xs, int zs, const double *m3, double h, double dt,
                        const double *src, int lsrc, int nt, int *field, long *idx, double *amp)
{
    double f = 1.0 / OR_PI / 1.4142135623731 / (h * h);
    double mxx = m3[0], mxz = m3[1], mzz = m3[2];
    if (kind == 1) { mxx = 1.0; mxz = 0.0; mzz = 1.0; }
    int nterm = 0;
#define OR_TERM(FLD, IX, IZ, SCALE)                                     \
    do {                                                                \
        field[nterm] = (FLD);                                           \
        idx[nterm] = (long)(IZ) * nx + (IX);                            \
        for (int it = 0; it < nt; it++) {                               \
            double s = 0.0;                                             \
            if (kind == 13) s = src[it < lsrc ? it : lsrc - 1];         \
            else if (it < lsrc) s = src[it];                            \
            amp[(long)nterm * nt + it] = (SCALE) * s;                   \
        }                                                               \
        nterm++;                                                        \
    } while (0)
    if (kind == 13) {
        double fp = f * dt / h;
        /* running sum of src, PD/main.cpp:106-111 */
        double *ps = (double *)malloc(sizeof(double) * (size_t)(lsrc > 0 ? lsrc : 1));
        double sum = 0.0;
        for (int i = 0; i < lsrc; i++) { sum += src[i]; ps[i] = sum; }
        const double *save = src;
        src = ps;
        OR_TERM(OR_TXX, xs, zs, -(mxx * fp));
        OR_TERM(OR_TXX, xs - 1, zs, (mxx * fp));
        OR_TERM(OR_TZZ, xs, zs, -(mzz * fp));
        OR_TERM(OR_TZZ, xs - 1, zs, (mzz * fp));
        for (int ixs = xs - 1; ixs <= xs; ixs++)
            for (int izs = zs; izs <= zs + 1; izs++) {
                OR_TERM(OR_TXZ, ixs, izs, -(mxz * fp * 0.25));
                OR_TERM(OR_TXZ, ixs - 1, izs, (mxz * fp * 0.25));
            }
        src = save;
        free(ps);
    } else {
        OR_TERM(OR_TXX, xs, zs, -(mxx * f));
        OR_TERM(OR_TZZ, xs, zs, -(mzz * f));
        if (mxz != 0.0 || kind != 1)
            for (int ixs = xs - 1; ixs <= xs; ixs++)
                for (int izs = zs; izs <= zs + 1; izs++) OR_TERM(OR_TXZ, ixs, izs, -(mxz * f * 0.25));
    }
    return nterm;
}

/* SH source terms, SH/point_source/cu_point_source.cu.
 *   kind 3  : moment (Mxy on Tx at xs,xs-1; Mzy on Tz at zs,zs+1), :6-66
 *   kind 13 : 'p' dipole form, :68-150
 *   kind 2  : line force on V at (xs,zs), :162-200
 * m2 = (Mxy, Mzy). */
int or_sh_source_terms(int kind, int nx, int xs, int zs, const double *m2, double h, double dt,
                       const double *src, int lsrc, int nt, int *field, long *idx, double *amp)
{
    double f = 1.0 / OR_PI / 1.4142135623731 / (h * h);
    double mxy = m2[0], mzy = m2[1];
    int nterm = 0;
    if (kind == 13) {
        double fp = f * dt / h;
        double *ps = (double *)malloc(sizeof(double) * (size_t)(lsrc > 0 ? lsrc : 1));
        double sum = 0.0;
        for (int i = 0; i < lsrc; i++) { sum += src[i]; ps[i] = sum; }
        const double *save = src;
        src = ps;
        OR_TERM(OR_TX, xs, zs, -(0.5 * mxy * fp));
        OR_TERM(OR_TX, xs - 1, zs, -(0.5 * mxy * fp));
        OR_TERM(OR_TZ, xs, zs, -(0.5 * mzy * fp));
        OR_TERM(OR_TZ, xs, zs + 1, -(0.5 * mzy * fp));
        OR_TERM(OR_TX, xs - 1, zs, (0.5 * mxy * fp));
        OR_TERM(OR_TX, xs - 2, zs, (0.5 * mxy * fp));
        OR_TERM(OR_TZ, xs - 1, zs, (0.5 * mzy * fp));
        OR_TERM(OR_TZ, xs - 1, zs + 1, (0.5 * mzy * fp));
        src = save;
        free(ps);
    } else if (kind == 2) {
        OR_TERM(OR_V, xs, zs, -(0.5 * mxy * f));
    } else {
        OR_TERM(OR_TX, xs, zs, -(0.5 * mxy * f));
        OR_TERM(OR_TX, xs - 1, zs, -(0.5 * mxy * f));
        OR_TERM(OR_TZ, xs, zs, -(0.5 * mzy * f));
        OR_TERM(OR_TZ, xs, zs + 1, -(0.5 * mzy * f));
    }
#undef OR_TERM
    return nterm;
}

/* ------------------------------------------------------------------------- */
/* Polygon model rasteriser, restating the semantics of PD/model/model.cpp:  */
/* get_elas_model (:175-237) and the ray-crossing test inside() (:437-469).  */
/* Polygon 0 is the background; later polygons overwrite earlier ones.       */
/* ------------------------------------------------------------------------- */
static int or_inside(double xp, double zp, const double *vx, const double *vz, int n)
{
    int nleft = 0;
    double x2 = vx[n - 1], z2 = vz[n - 1];
    for (int j = 0; j < n; j++) {
        double x1 = x2, z1 = z2;
        x2 = vx[j];
        z2 = vz[j];
        double zmin = z1 < z2 ? z1 : z2, zmax = z1 > z2 ? z1 : z2;
        if (zmin >= zp) continue;
        if (zmax < zp) continue;
        if (z1 == z2) { /* horizontal edge at the query depth */
            double xmax = x1 > x2 ? x1 : x2, xmin = x1 < x2 ? x1 : x2;
            if (xp > xmax) continue;
            if (xp >= xmin) return 1;
            nleft++;
            continue;
        }
        double xi = x1 + (zp - z1) * (x2 - x1) / (z2 - z1);
        if (xi == xp) return 1;
        if (xi > xp) nleft++;
    }
    return nleft % 2;
}

void or_mdl_raster(int nx, int nz, double h, int npoly, const int *nvert, const double *vx,
                   const double *vz, const double *pvp, const double *pvs, const double *pden,
                   double *vp, double *vs, double *den)
{
    const long n = (long)nx * nz;
    for (long k = 0; k < n; k++) { vp[k] = pvp[0]; vs[k] = pvs[0]; den[k] = pden[0]; }
    long off = nvert[0];
    for (int p = 1; p < npoly; p++) {
        const double *px = vx + off, *pz = vz + off;
        int nv = nvert[p];
        off += nv;
        double x1 = 1e28, x2 = -1e28, z1 = 1e28, z2 = -1e28;
        for (int j = 0; j < nv; j++) {
            if (px[j] < x1) x1 = px[j];
            if (px[j] > x2) x2 = px[j];
            if (pz[j] < z1) z1 = pz[j];
            if (pz[j] > z2) z2 = pz[j];
        }
        int ix1 = (int)(x1 / h - 1), ix2 = (int)(x2 / h + 1);
        int iz1 = (int)(z1 / h - 1), iz2 = (int)(z2 / h + 1);
#define OR_CLAMP(v, hi) v = (v) < 0 ? 0 : ((v) > (hi) ? (hi) : (v))
        OR_CLAMP(ix1, nx - 1); OR_CLAMP(ix2, nx - 1);
        OR_CLAMP(iz1, nz - 1); OR_CLAMP(iz2, nz - 1);
#undef OR_CLAMP
        for (int iz = iz1; iz <= iz2; iz++)
            for (int ix = ix1; ix <= ix2; ix++) {
                double xp = h * (double)ix, zp = h * (double)iz;
                if (or_inside(xp, zp, px, pz, nv)) {
                    long k = (long)iz * nx + ix;
                    vp[k] = pvp[p]; vs[k] = pvs[p]; den[k] = pden[p];
                }
            }
    }
}

/* ------------------------------------------------------------------------- */
/* Time stepping, instantiated for double and float.                         */
/* ------------------------------------------------------------------------- */
#define REAL double
#define FMA fma
#define SFX f64
#include "fd23_oracle_step.inc"
#undef REAL
#undef FMA
#undef SFX

#define REAL float
#define FMA fmaf
#define SFX f32
#include "fd23_oracle_step.inc"
#undef REAL
#undef FMA
#undef SFX

int or_version(void) { return 1; }
