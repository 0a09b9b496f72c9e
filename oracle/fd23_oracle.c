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
/* Hybrid box, host side.                                                    */
/* ------------------------------------------------------------------------- */

/* Ring sizes of a bx x bz box (both >= 16): the sub ring is the outer 4 cells
 * of the box (PD/box/box.cpp:59-76: s0..s7 minus the open interior (s1, s6)),
 * the add ring the next 4 cells inward (box.cpp:78-95: s2..s5 minus (s3, s4)).
 * Returns nsub + nadd, or -1. */
int or_box_ring_count(int bx, int bz, int *nsub, int *nadd)
{
    if (bx < 16 || bz < 16) return -1;
    *nsub = 8 * (bx + bz - 8);
    *nadd = 8 * (bx + bz - 24);
    return *nsub + *nadd;
}

/* Ring cells in incident-field order: the sub ring row by row, then the add
 * ring row by row (the loops of box.cpp:59-95).  gidx = row-major grid index
 * (nx columns), ridx = row-major box index.  Returns nsub + nadd or -1. */
int or_box_rings(int nx, int x0, int z0, int bx, int bz, long *gidx, long *ridx, int *nsub, int *nadd)
{
    if (or_box_ring_count(bx, bz, nsub, nadd) < 0) return -1;
    int k = 0;
    for (int j = 0; j < bz; j++)
        for (int i = 0; i < bx; i++)
            if (!(i > 3 && i < bx - 4 && j > 3 && j < bz - 4)) {
                ridx[k] = (long)j * bx + i;
                gidx[k] = (long)(j + z0) * nx + (i + x0);
                k++;
            }
    for (int j = 4; j < bz - 4; j++)
        for (int i = 4; i < bx - 4; i++)
            if (!(i > 7 && i < bx - 8 && j > 7 && j < bz - 8)) {
                ridx[k] = (long)j * bx + i;
                gidx[k] = (long)(j + z0) * nx + (i + x0);
                k++;
            }
    return k;
}

/* Incident field on the ring cells from two displacement planes, restating
 * BOX::setboxsource (PD/box/box.cpp:120-196) for a bx x bz box.  Planes are
 * (bx+8) x (bz+8), row-major, box cell (i, j) at plane (i+4, j+4); uo / wo
 * are the planes of this step, un / wn of the next.  rmat = box material
 * LAM, MU, MUA (dt/h scaled, bx*bz each).  Output [U W Txx Txz Tzz][nring]:
 *   U = (un - uo)/dt,  W = (wn - wo)/dt,
 *   Txx = (GAM*ux + LAM*wz)/dt, Tzz = (LAM*ux + GAM*wz)/dt, Txz = MUA*(wx+uz)/dt
 * with derivatives of the new planes at the reduced order
 *   ord = max(0, min(4, max(|ty-3-(bz+1)/2| - 1, |tx-3-(bx+1)/2| - 1)))
 * (the reference's square-box formula per axis).  Expressions are evaluated
 * left to right as written in the reference. */
int or_box_incident_from_displacement(int bx, int bz, double dt, const double *rmat, const double *uo,
                                      const double *wo, const double *un, const double *wn, double *out)
{
    int nsub, nadd;
    const int nring = or_box_ring_count(bx, bz, &nsub, &nadd);
    if (nring < 0) return -1;
    const long nb = (long)bx * bz;
    const int pw = bx + 8;
    const double *LAM = rmat, *MU = rmat + nb, *MUA = rmat + 2 * nb;
    long *gidx = (long *)malloc(sizeof(long) * nring), *ridx = (long *)malloc(sizeof(long) * nring);
    if (!gidx || !ridx) {
        free(gidx);
        free(ridx);
        return -1;
    }
    or_box_rings(bx, 0, 0, bx, bz, gidx, ridx, &nsub, &nadd);
#define PL(a, i, j) (a)[(long)(i) + (long)(j) * pw]
    for (int q = 0; q < nring; q++) {
        const int bi = (int)(ridx[q] % bx), bj = (int)(ridx[q] / bx);
        const int tx = bi + 4, ty = bj + 4;
        int oz = abs(ty - 3 - (bz + 1) / 2) - 1, ox = abs(tx - 3 - (bx + 1) / 2) - 1;
        int ord = oz > ox ? oz : ox;
        if (ord > 4) ord = 4;
        if (ord < 0) ord = 0;
        const double *c = OR_COEF[ord];
        const double ux = c[0] * (PL(un, tx, ty) - PL(un, tx - 1, ty)) - c[1] * (PL(un, tx + 1, ty) - PL(un, tx - 2, ty)) +
                          c[2] * (PL(un, tx + 2, ty) - PL(un, tx - 3, ty)) - c[3] * (PL(un, tx + 3, ty) - PL(un, tx - 4, ty));
        const double uz = c[0] * (PL(un, tx, ty) - PL(un, tx, ty - 1)) - c[1] * (PL(un, tx, ty + 1) - PL(un, tx, ty - 2)) +
                          c[2] * (PL(un, tx, ty + 2) - PL(un, tx, ty - 3)) - c[3] * (PL(un, tx, ty + 3) - PL(un, tx, ty - 4));
        const double wx = c[0] * (PL(wn, tx + 1, ty) - PL(wn, tx, ty)) - c[1] * (PL(wn, tx + 2, ty) - PL(wn, tx - 1, ty)) +
                          c[2] * (PL(wn, tx + 3, ty) - PL(wn, tx - 2, ty)) - c[3] * (PL(wn, tx + 4, ty) - PL(wn, tx - 3, ty));
        const double wz = c[0] * (PL(wn, tx, ty + 1) - PL(wn, tx, ty)) - c[1] * (PL(wn, tx, ty + 2) - PL(wn, tx, ty - 1)) +
                          c[2] * (PL(wn, tx, ty + 3) - PL(wn, tx, ty - 2)) - c[3] * (PL(wn, tx, ty + 4) - PL(wn, tx, ty - 3));
        const long b = ridx[q];
        const double lam = LAM[b], mu = MU[b], mua = MUA[b];
        const double gam = lam + 2.0 * mu;
        out[0L * nring + q] = (PL(un, tx, ty) - PL(uo, tx, ty)) / dt;
        out[1L * nring + q] = (PL(wn, tx, ty) - PL(wo, tx, ty)) / dt;
        out[2L * nring + q] = (gam * ux + lam * wz) / dt;
        out[3L * nring + q] = (mua * (wx + uz)) / dt;
        out[4L * nring + q] = (lam * ux + gam * wz) / dt;
    }
#undef PL
    free(gidx);
    free(ridx);
    return nring;
}

/* Box material cut from the full (dt/h scaled) material, restating
 * MATERIAL::init_for_box_from_full (PD/material/material.cpp:39-97): every box
 * cell whose BU, BW differ from b = dt/(h*srcden), MU, MUA from
 * mu = srcvs^2*srcden*dt/h, or LAM from lam = (srcvp^2*srcden - 2 mu)*dt/h by
 * more than 1e-4 relative is set to the homogeneous values IN THE FULL
 * material; the box copy follows.  mat / rmat: LAM MU MUA BU BW.  Returns the
 * number of cells replaced. */
int or_box_material(int nx, int nz, double *mat, int x0, int z0, int bx, int bz, double srcvp, double srcvs,
                    double srcden, double dt, double h, double *rmat)
{
    const long n = (long)nx * nz, nb = (long)bx * bz;
    double mu = srcvs * srcvs * srcden;
    double lam = (srcvp * srcvp * srcden - 2.0 * mu);
    double b = 1.0 / srcden;
    mu = mu * dt / h;
    lam = lam * dt / h;
    b = b * dt / h;
    const double eps = 1E-4;
    double *LAM = mat, *MU = mat + n, *MUA = mat + 2 * n, *BU = mat + 3 * n, *BW = mat + 4 * n;
    int nrep = 0;
    for (int j = 0; j < bz; j++)
        for (int i = 0; i < bx; i++) {
            const long g = (long)(i + x0) + (long)(j + z0) * nx, k = (long)i + (long)j * bx;
            if (fabs(b - BU[g]) > b * eps || fabs(b - BW[g]) > b * eps || fabs(mu - MU[g]) > mu * eps ||
                fabs(mu - MUA[g]) > mu * eps || fabs(lam - LAM[g]) > lam * eps) {
                BU[g] = b;
                BW[g] = b;
                MU[g] = mu;
                MUA[g] = mu;
                LAM[g] = lam;
                nrep++;
            }
            rmat[k] = LAM[g];
            rmat[nb + k] = MU[g];
            rmat[2 * nb + k] = MUA[g];
            rmat[3 * nb + k] = BU[g];
            rmat[4 * nb + k] = BW[g];
        }
    return nrep;
}


/* ------------------------------------------------------------------------- */
/* Time stepping, instantiated for double and float.                         */
/* ------------------------------------------------------------------------- */
/* ---- usepunch: tile step windows ----
 * PD/slide/cu_slide.cu:6-66 turns a travel-time file into per-tile steps
 * first = int((tmin - before)/dt), last = int((tmax + after)/dt) over tiles of
 * BDIMX x BDIMY = 32 x 16 cells (PD/param/const.h:20-21); the sweep kernels
 * return at once for a cell whose tile has it <= first or it >= last
 * (CHECK_IF_NEED_UPDATE, PD/fd/cu_fd.cu:16-23, at :249 and :404).  The
 * windows are installed for the next runs by or_set_punch (NULL: none);
 * tiles are counted ceil(nx/32) per row. */
static const int *or_pfirst = NULL, *or_plast = NULL;
static int or_pnbx = 0;

void or_set_punch(const int *first, const int *last, int nbx)
{
    or_pfirst = first;
    or_plast = last;
    or_pnbx = nbx;
}

static inline int or_punch_skip(int nx, int ix, int iz, int it)
{
    (void)nx;
    if (!or_pfirst) return 0;
    const long t = (long)(iz / 16) * or_pnbx + ix / 32;
    return it <= or_pfirst[t] || it >= or_plast[t];
}

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

/* FP32 with every multiply-add rounded twice (a product, then a sum): what a
 * build without multiply-add contraction computes, e.g. the reference's FP32
 * program built for device debugging (nvcc -G; PSV/clean_nobox/Makefile).
 * Used to test whether the reference's FP32 restart states
 * (PSV/clean_nobox/TEST/tt) came from such a build; -ffp-contract=off keeps
 * the two roundings. */
static inline float or_mul_add_f(float a, float b, float c)
{
    const float p = a * b;
    return p + c;
}
#define REAL float
#define FMA or_mul_add_f
#define SFX f32nf
#include "fd23_oracle_step.inc"
#undef REAL
#undef FMA
#undef SFX

/* ------------------------------------------------------------------------- */
/* Box-source generator (FP64): the ntde_line program,                        */
/* PD/source/source_line.cpp:307-410 (main), :196-305                         */
/* (compute_pQpW_mathematica) and the wavelet convolution cu_con of           */
/* PD/source/cu_source.cu:2-42.                                               */
/* ------------------------------------------------------------------------- */

/* Radiation coefficients A1, A2, A3 of a line moment source
 * (PD/source/source_line.cpp:320-326): theta = azimuth - strike, delta = dip,
 * lambda = rake, degrees. */
void or_line_source_coefs(double strike, double dip, double rake, double azimuth, double *a)
{
    const double d = dip * OR_PI / 180.0, l = rake * OR_PI / 180.0, th = (azimuth - strike) * OR_PI / 180.0;
    a[0] = sin(2.0 * th) * cos(l) * sin(d) + 0.5 * cos(2.0 * th) * sin(l) * sin(2.0 * d);
    a[1] = cos(th) * cos(l) * cos(d) - sin(th) * sin(l) * cos(2.0 * d);
    a[2] = 0.5 * sin(l) * sin(2.0 * d);
}

/* Per receiver point (r, z) (metres from the source, z down) and component
 * (0 = horizontal "Q", 1 = vertical "W"), the time derivative of the 2-D
 * full-space displacement of the line source is
 *   v(t) = t^3 (Ta - Tb) k[0] + t (Ta k[1] + Tb k[2]) + (Ta k[3] + Tb k[4]) / t
 * with Ta = 1/sqrt(1 - (R/(t vp))^2), Tb likewise with vs.  k[] folds the
 * closed-form polynomials in r and z of the reference expressions
 * (source_line.cpp:262-299, one table row per radiation term A1, A2, A3 and
 * per power of t), the radiation coefficients, 1/vp^2, 1/vs^2, 1/vp^4,
 * 1/vs^4 and G/R^8, G = sqrt(2)/(4 pi^2 den).  Products and sums in the order
 * written; the CUDA generator evaluates the same sequence. */
void or_line_source_kcoef(double r, double z, int comp, double vp, double vs, double den, const double *a,
                          double *k)
{
    const double r2 = r * r, z2 = z * z, rz = r * z;
    const double r4 = r2 * r2, z4 = z2 * z2, r6 = r4 * r2, z6 = z4 * z2, z8 = z4 * z4;
    const double R2 = r2 + z2, R4 = R2 * R2;
    const double dif = r2 - z2;
    const double e4 = r4 - 6.0 * r2 * z2 + z4;                   /* r^4 - 6 r^2 z^2 + z^4 */
    const double e6 = r6 - 5.0 * r4 * z2 - 5.0 * r2 * z4 + z6;   /* r^6 - 5 r^4 z^2 - 5 r^2 z^4 + z^6 */
    const double f4 = 3.0 * r4 - 2.0 * r2 * z2 - 5.0 * z4;       /* 3 r^4 - 2 r^2 z^2 - 5 z^4 */
    double p[3][5]; /* [A term][t^3, t*Ta, t*Tb, Ta/t, Tb/t] */
    if (comp == 0) {
        p[0][0] = e4;
        p[0][1] = 2.0 * (3.0 * r4 * z2 + 2.0 * r2 * z4 - z6);
        p[0][2] = e6;
        p[0][3] = R4 * z4;
        p[0][4] = r2 * R4 * z2;
        p[1][0] = -8.0 * rz * dif;
        p[1][1] = 2.0 * rz * f4;
        p[1][2] = 8.0 * rz * (z4 - r4);
        p[1][3] = 2.0 * rz * R4 * z2;
        p[1][4] = rz * R4 * dif;
        p[2][0] = -3.0 * e4;
        p[2][1] = 2.0 * (r6 - 8.0 * r4 * z2 - 7.0 * r2 * z4 + 2.0 * z6);
        p[2][2] = -3.0 * e6;
        p[2][3] = 2.0 * r6 * z2 + 3.0 * r4 * z4 - z8;
        p[2][4] = -3.0 * r2 * R4 * z2;
    } else {
        p[0][0] = 4.0 * rz * dif;
        p[0][1] = -rz * f4;
        p[0][2] = rz * f4;
        p[0][3] = -rz * R4 * z2;
        p[0][4] = rz * R4 * z2;
        p[1][0] = 2.0 * e4;
        p[1][1] = -2.0 * e6;
        p[1][2] = r6 - 11.0 * r4 * z2 - 9.0 * r2 * z4 + 3.0 * z6;
        p[1][3] = -2.0 * r2 * R4 * z2;
        p[1][4] = R4 * dif * z2;
        p[2][0] = -12.0 * rz * dif;
        p[2][1] = rz * (13.0 * r4 + 2.0 * r2 * z2 - 11.0 * z4);
        p[2][2] = -3.0 * rz * f4;
        p[2][3] = rz * (z6 - 2.0 * r6 - 3.0 * r4 * z2);
        p[2][4] = -3.0 * rz * R4 * z2;
    }
    const double ivp2 = 1.0 / (vp * vp), ivs2 = 1.0 / (vs * vs);
    const double G = sqrt(2.0) / (4.0 * OR_PI * OR_PI * den);
    const double S = G / (R4 * R4);
    const double w[5] = {S, S * ivp2, S * ivs2, S * (ivp2 * ivp2), S * (ivs2 * ivs2)};
    for (int j = 0; j < 5; j++) k[j] = (a[0] * p[0][j] + a[1] * p[1][j] + a[2] * p[2][j]) * w[j];
}

/* The wave factor T(i) at sample i (t = i dt) for travel time R/v
 * (source_line.cpp:199-222): 0 up to the arrival step n = floor(R/v/dt);
 * at n+1 the integrated first sample sqrt(b (2 R/(v dt) + b)),
 * b = (n+1) - R/v/dt + 0.5; afterwards 1/sqrt(1 - (R/(t v))^2). */
static double or_line_wave(double R, double v, double dt, int i)
{
    const double u = R / v / dt;
    const int n = (int)floor(u);
    if (i <= n) return 0.0;
    if (i == n + 1) {
        const double b = ((double)(n + 1) - u) + 0.5;
        return sqrt(b * (2.0 * u + b));
    }
    const double t = i * dt, q = R / (t * v);
    return 1.0 / sqrt(1.0 - q * q);
}

/* One sample of v(t) above; samples before the P arrival step are 0 (the
 * arrival step itself is evaluated, which at t = 0 gives 0/0 as in the
 * reference). */
double or_line_sample(double R, const double *k, double vp, double vs, double dt, int i)
{
    const int na = (int)floor(R / vp / dt);
    if (i < na) return 0.0;
    const double t = i * dt;
    const double ta = or_line_wave(R, vp, dt, i), tb = or_line_wave(R, vs, dt, i);
    const double t3 = (t * t) * t;
    double v = (t3 * (ta - tb)) * k[0];
    v = v + t * (ta * k[1] + tb * k[2]);
    v = v + (ta * k[3] + tb * k[4]) / t;
    return v;
}

/* Displacement planes of frames it0 .. it0+nf-1: out[f][comp][q*px + p],
 * comp 0 = U plane (point ((ox+p)+0.5-sx, (oz+q)-sz) cells from the source),
 * comp 1 = W plane (point ((ox+p)-sx, (oz+q)-0.5-sz)); both times h.  Each
 * sample is the causal convolution with the wavelet src[0..lsrc) in the
 * reference kernel's order: the wavelet padded with zeros to a multiple of
 * 32 taps, taps taken from the last to the first, one fused multiply-add
 * each (PD/source/cu_source.cu:2-16; out[k] = sum_j src[j] g[k-j], g = 0
 * before sample 0).  The reference program writes frames 0 .. nt-1 for the
 * square box px = pz = bw+8, ox = oz = (bw+1)/2 + 4 + 1 - (bw+8),
 * sx = 0.25, sz = -0.25.  Returns 0, -1 on bad arguments or memory. */
int or_line_source_planes(int px, int pz, int ox, int oz, double h, double dt, double vp, double vs, double den,
                          const double *a, double sx, double sz, const double *src, int lsrc, int it0, int nf,
                          double *out)
{
    if (px <= 0 || pz <= 0 || lsrc <= 0 || it0 < 0 || nf < 0 || !(vp > 0) || !(vs > 0) || !(dt > 0)) return -1;
    const int ntap = ((lsrc + 31) / 32) * 32;
    const int ng = it0 + nf; /* samples 0 .. ng-1 of g */
    double *tap = (double *)calloc((size_t)ntap, sizeof(double));
    double *g = (double *)malloc(sizeof(double) * (size_t)(ng > 0 ? ng : 1));
    if (!tap || !g) {
        free(tap);
        free(g);
        return -1;
    }
    for (int j = 0; j < lsrc; j++) tap[j] = src[j];
    const long plane = (long)px * pz;
    for (int comp = 0; comp < 2; comp++)
        for (int q = 0; q < pz; q++)
            for (int p = 0; p < px; p++) {
                const double x = comp == 0 ? ((ox + p) + 0.5) - sx : (ox + p) - sx;
                const double zz = comp == 0 ? (oz + q) - sz : ((oz + q) - 0.5) - sz;
                const double r = x * h, z = zz * h;
                double k[5];
                or_line_source_kcoef(r, z, comp, vp, vs, den, a, k);
                const double R = sqrt(r * r + z * z);
                for (int i = 0; i < ng; i++) g[i] = or_line_sample(R, k, vp, vs, dt, i);
                for (int f = 0; f < nf; f++) {
                    const int it = it0 + f;
                    double acc = 0.0;
                    for (int j = ntap - 1; j >= 0; j--) acc = fma(tap[j], it - j >= 0 ? g[it - j] : 0.0, acc);
                    out[((long)f * 2 + comp) * plane + (long)q * px + p] = acc;
                }
            }
    free(tap);
    free(g);
    return 0;
}

int or_version(void) { return 1; }
