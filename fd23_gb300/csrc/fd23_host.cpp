// Host-side FP64 set-up for the fd23 engine: material, CPML profiles,
// wavelets, moment tensors, point-source injection terms and receiver lists.
//
// These run once per shot on the CPU in double precision, exactly as the
// reference does, and are compiled with -ffp-contract=off so that x86 and
// Arm hosts produce the same bits.  Reference paths are relative to the fd23
// project root (PD = PSV/psv_clean_double, PN = PSV/clean_nobox, SH = SH).
#include "fd23_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

namespace fd23 {

// 8th-order staggered-grid coefficient rows for stencil order 0..4
// (PD/param/const.h:1-19).  Rows 0 and 1 are the same 2nd-order pair.
const double kCoef[5][4] = {
    {1.0, 0.0, 0.0, 0.0},
    {1.0, 0.0, 0.0, 0.0},
    {9.0 / 8.0, 1.0 / 24.0, 0.0, 0.0},
    {75.0 / 64.0, 25.0 / 384.0, 3.0 / 640.0, 0.0},
    {1225.0 / 1024.0, 245.0 / 3072.0, 49.0 / 5120.0, 5.0 / 7168.0}};

static const double kPi = 3.14159265358979;  // PD/param/const.h:26

double cfl_number(double vmax, double h, double dt)
{
    // stab = vmax*dt*sum(E)*sqrt(2)/h, PD/material/material.cpp:296-301
    const double esum = kCoef[4][0] + kCoef[4][1] + kCoef[4][2] + kCoef[4][3];
    return vmax * dt * esum * std::sqrt(2.0) / h;
}

// P-SV material: LAM, MU, MUA, BU, BW.  Edge rules of
// PD/material/material.cpp:156-282, in order:
//   1. mu = vs^2 rho, lam = vp^2 rho - 2 mu
//   2. fluid cells (vs/vp < 0.01) within 5 cells of the left, right and
//      bottom edges get mu = vp^2 rho / 3 (a stabiliser for water edges)
//   3. rows >= 1: BU, BW harmonic-mean buoyancies and MUA, the 4-point
//      harmonic shear average (its denominator counts m2*m3*m4 twice, as the
//      reference does); BU's right neighbour of the last column is the first
//      cell of the next row; BW of the last row pairs the cell with itself
//   4. row 0 (free surface, Mittet 2002) for 1 <= ix <= nx-2:
//      BU = 4/(rho+rho_right), LAM = 0, MU /= 2
//   5. everything times dt/h
int build_psv_material(int nx, int nz, double h, double dt, const double *vp, const double *vs,
                       const double *den, double *out, double *stab)
{
    const long n = (long)nx * nz;
    double *lamA = out, *muA = out + n, *muaA = out + 2 * n, *buA = out + 3 * n,
           *bwA = out + 4 * n;
    std::fill(out, out + 5 * n, 0.0);
    for (long k = 0; k < n; ++k) {
        const double mu = vs[k] * vs[k] * den[k];
        muA[k] = mu;
        lamA[k] = vp[k] * vp[k] * den[k] - 2.0 * mu;
    }
    auto fluid_fix = [&](long k) {
        if (vs[k] / vp[k] < 0.01) {
            const double mu = vp[k] * vp[k] / 3.0 * den[k];
            muA[k] = mu;
            lamA[k] = vp[k] * vp[k] * den[k] - 2.0 * mu;
        }
    };
    const int band = 5;
    for (int iz = 0; iz < nz; ++iz) {
        for (int ix = 0; ix < std::min(band, nx); ++ix) fluid_fix((long)iz * nx + ix);
        for (int ix = std::max(nx - band, 0); ix < nx; ++ix) fluid_fix((long)iz * nx + ix);
    }
    for (int iz = std::max(nz - band, 0); iz < nz; ++iz)
        for (int ix = 0; ix < nx; ++ix) fluid_fix((long)iz * nx + ix);

    for (int iz = 1; iz < nz; ++iz) {
        for (int ix = 0; ix < nx; ++ix) {
            const long k = (long)iz * nx + ix;
            const long kr = (k + 1 < n) ? k + 1 : k;
            buA[k] = 2.0 / (den[k] + den[kr]);
            const long kb = (k + nx < n) ? k - nx : k;
            bwA[k] = 2.0 / (den[k] + den[kb]);
            if (ix + 1 < nx && iz + 1 < nz) {
                const double m1 = muA[k], m2 = muA[k + 1], m3 = muA[k - nx], m4 = muA[k + 1 - nx];
                const double d = std::max(m2 * m3 * m4 + m1 * m3 * m4 + m1 * m2 * m4 + m2 * m3 * m4,
                                          1e-10);
                muaA[k] = 4.0 * m1 * m2 * m3 * m4 / d;
            } else {
                muaA[k] = muA[k];
            }
        }
    }
    for (int ix = 1; ix < nx - 1; ++ix) {
        buA[ix] = 4.0 / (den[ix] + den[ix + 1]);
        lamA[ix] = 0.0;
        muA[ix] = 0.5 * muA[ix];
    }
    const double fac = dt / h;
    for (long k = 0; k < 5 * n; ++k) out[k] *= fac;

    double vmax = -99999.0;
    for (long k = 0; k < n; ++k) vmax = std::max(vmax, vp[k]);
    const double s = cfl_number(vmax, h, dt);
    if (stab) *stab = s;
    return s > 1.0 ? FD23_ERR_UNSTABLE : FD23_OK;
}

// SH material: MUX, MUZ (harmonic shear means with the right / upper
// neighbour, the first row and last cell pairing with themselves) and
// BV = 1/rho, all times dt/h.  SH/material/material.cpp:75-105, CFL on vs.
int build_sh_material(int nx, int nz, double h, double dt, const double *vs, const double *den,
                      double *out, double *stab)
{
    const long n = (long)nx * nz;
    double *muxA = out, *muzA = out + n, *bvA = out + 2 * n;
    auto shear = [&](long k) { return vs[k] * vs[k] * den[k]; };
    auto harm = [](double a, double b) { return 2.0 * a * b / std::max(a + b, 1e-10); };
    for (long k = 0; k < n; ++k) {
        bvA[k] = 1.0 / den[k];
        const double m1 = shear(k);
        muxA[k] = harm(m1, (k + 1 < n) ? shear(k + 1) : m1);
        muzA[k] = harm(m1, (k - nx >= 0) ? shear(k - nx) : m1);
    }
    const double fac = dt / h;
    for (long k = 0; k < 3 * n; ++k) out[k] *= fac;
    double vmax = -99999.0;
    for (long k = 0; k < n; ++k) vmax = std::max(vmax, vs[k]);
    const double s = cfl_number(vmax, h, dt);
    if (stab) *stab = s;
    return s > 1.0 ? FD23_ERR_UNSTABLE : FD23_OK;
}

// One CPML profile (b, c, k) along an axis of n points, PD/cpml/cpml.cpp:7-83.
// Damping d = distance into the layer / npml (cells, staggered by start),
// sigma = sigmax d^2, kappa = 1 + d^2, alpha = pi fc (1 - d),
// b = exp(-(sigma/kappa + alpha) pml_dt), c = sigma (b-1) / (sigma + kappa alpha) / kappa,
// k = 1/kappa; the 4 first and 5 last points are frozen to zero.
void build_cpml_profile(int npml, double start, int n, double pml_dt, double pml_r, double pml_v,
                        double pml_fc, double *b, double *c, double *k)
{
    const double edge = npml - 0.5;
    const double sigmax = -3.0 / (2.0 * std::floor(edge)) * pml_v * std::log(pml_r);
    const double alphamax = 3.141592653589 * pml_fc;
    std::vector<double> d((size_t)n, 0.0);
    for (int i = 0; i < std::min(npml + 2, n); ++i) {
        const double t = (edge - (i + start)) / std::floor((double)npml);
        if (t > 0) d[i] = t;
    }
    for (int i = std::max(n - npml - 2, 0); i < n; ++i) {
        const double t = ((i + start) - (n - 1 - edge)) / std::floor((double)npml);
        if (t > 0) d[i] = t;
    }
    for (int i = 0; i < n; ++i) {
        const double sg = sigmax * std::pow(d[i], 2.0);
        const double kp = 1.0 + (2.0 - 1.0) * std::pow(d[i], 2.0);
        const double al = alphamax * (1.0 - std::pow(d[i], 1.0));
        const double bb = std::exp(-(sg / kp + al) * pml_dt);
        b[i] = bb;
        c[i] = (sg + kp * al < 1e-15) ? 0.0 : sg * (bb - 1.0) / (sg + kp * al) / kp;
        k[i] = 1.0 / kp;
    }
    for (int i = 0; i < n; ++i)
        if (i < 4 || i >= n - 5) b[i] = c[i] = k[i] = 0.0;
}

// Full coefficient set in b|c|k block order (see fd23.h).  Staggered start
// offsets: P-SV PD/cpml/cpml.cpp:177-185, SH SH/cpml/cpml.cpp:172-176.
void build_cpml(int wave, int nx, int nz, int npml, double pml_dt, double pml_r, double pml_v,
                double pml_fc, std::vector<double> &bck)
{
    struct Comp { double start; bool along_x; };
    std::vector<Comp> comps;
    if (wave == FD23_PSV)
        comps = {{0.5, true}, {0.0, true}, {0.0, true}, {0.5, true},     // Txx_x Txz_x U_x W_x
                 {0.0, false}, {0.5, false}, {0.0, false}, {0.5, false}}; // Tzz_z Txz_z U_z W_z
    else
        comps = {{0.0, true}, {0.5, true}, {0.5, false}, {0.0, false}};  // Tx_x V_x Tz_z V_z
    size_t blk = 0;
    for (auto &c : comps) blk += c.along_x ? nx : nz;
    bck.assign(3 * blk, 0.0);
    size_t off = 0;
    for (auto &c : comps) {
        const int n = c.along_x ? nx : nz;
        build_cpml_profile(npml, c.start, n, pml_dt, pml_r, pml_v, pml_fc, &bck[off],
                           &bck[blk + off], &bck[2 * blk + off]);
        off += n;
    }
}

void moment_psv(double strike, double dip, double rake, double azimuth, double m[3])
{
    // PD/point_source/cu_point_source.cu:16-26
    const double dl = dip * kPi / 180.0, lb = rake * kPi / 180.0;
    const double ph = (strike - azimuth) * kPi / 180.0;
    m[0] = -(std::sin(dl) * std::cos(lb) * std::sin(2.0 * ph) +
             std::sin(2.0 * dl) * std::sin(lb) * std::sin(ph) * std::sin(ph));
    m[1] = -(std::cos(dl) * std::cos(lb) * std::cos(ph) +
             std::cos(2.0 * dl) * std::sin(lb) * std::sin(ph));
    m[2] = std::sin(2.0 * dl) * std::sin(lb);
}

void moment_sh(double strike, double dip, double rake, double azimuth, double m[2])
{
    // SH/point_source/cu_point_source.cu:16-24
    const double dl = dip * kPi / 180.0, lb = rake * kPi / 180.0;
    const double ph = (strike - azimuth) * kPi / 180.0;
    m[0] = std::sin(dl) * std::cos(lb) * std::cos(2.0 * ph) +
           0.5 * std::sin(2.0 * dl) * std::sin(lb) * std::sin(2.0 * ph);
    m[1] = -(std::cos(dl) * std::cos(lb) * std::sin(ph) -
             std::cos(2.0 * dl) * std::sin(lb) * std::cos(ph));
}

int wavelet_gaussian(double dt, int alpha, double *out, int cap)
{
    // PD/source/waveform.cpp:27-47: alpha < 0 normalised one-sided bell,
    // alpha >= 0 the odd function i*exp(-i^2/alpha^2); values are s(t)*dt.
    (void)dt;
    const int half = std::abs((int)(alpha * 3.0));
    const int len = 2 * half + 1;
    if (!out || cap < len) return FD23_ERR_ARG;
    const double a2 = (double)alpha * alpha;
    if (alpha >= 0) {
        for (int i = -half; i <= half; ++i) out[i + half] = (double)i * std::exp((double)(-i) * (double)i / a2);
    } else {
        double sum = 0.0;
        for (int i = -half; i <= half; ++i) {
            out[i + half] = std::exp((double)(-i) * (double)i / a2);
            sum += out[i + half];
        }
        for (int i = 0; i < len; ++i) out[i] /= sum;
    }
    return len;
}

int wavelet_trapezoid(double dt, double t1, double t2, double t3, double *out, int cap)
{
    // PD/source/waveform.cpp:8-25
    const int n1 = (int)(t1 / dt), n3 = (int)(t3 / dt);
    const int n2 = (int)(t2 / dt) + n1;
    const int len = n2 + n3;
    if (!out || cap < len) return FD23_ERR_ARG;
    const double amp = (t2 + 0.5 * (t1 + t3)) / dt;
    int p = 0, i = 0;
    for (; i < n1; ++i) out[p++] = i / (n1 * amp);
    for (; i < n2; ++i) out[p++] = 1.0 / amp;
    for (i = n3; i > 0; --i) out[p++] = i / (n3 * amp);
    return len;
}

int wavelet_ricker(double dt, double f0, double t0, double *out, int cap)
{
    // not in the reference: (1 - 2 a) exp(-a), a = (pi f0 (t - t0))^2,
    // sampled at t = i*dt and stored as s(t)*dt like the reference wavelets
    if (f0 <= 0 || dt <= 0) return FD23_ERR_ARG;
    if (t0 <= 0) t0 = 1.2 / f0;
    const int len = (int)std::lround(2.0 * t0 / dt) + 1;
    if (!out || cap < len) return FD23_ERR_ARG;
    for (int i = 0; i < len; ++i) {
        const double t = i * dt - t0;
        const double a = (M_PI * f0 * t) * (M_PI * f0 * t);
        out[i] = (1.0 - 2.0 * a) * std::exp(-a) * dt;
    }
    return len;
}

// Point-source injection terms (field, ix, iz, per-step amplitude).  The
// amplitude of step it is scale*s(it) with s the wavelet (kind 3, 2, 1: zero
// after lsrc) or its running sum clamped at the last sample (kind 13).
// Terms and their order follow PD/point_source/cu_point_source.cu:38-63
// (kind 3), :117-159 (kind 13), PN/point_source/cu_point_source.cu:16-20
// (explosion), SH/point_source/cu_point_source.cu:37-64 (SH), :68-150 (SH
// 'p') and :162-200 (SH force).
void build_source_terms(int wave, int kind, int xs, int zs, const double *moment, double h,
                        double dt, const double *src, int lsrc, int nt,
                        std::vector<SourceTerm> &terms, std::vector<double> &amp)
{
    terms.clear();
    amp.clear();
    const double f = 1.0 / kPi / 1.4142135623731 / (h * h);
    std::vector<double> wav(src, src + lsrc);
    if (kind == FD23_SRC_MOMENT_P) {
        double run = 0.0;
        for (auto &v : wav) { run += v; v = run; }
    }
    auto sample = [&](int it) -> double {
        if (lsrc <= 0) return 0.0;
        if (kind == FD23_SRC_MOMENT_P) return wav[std::min(it, lsrc - 1)];
        return it < lsrc ? wav[it] : 0.0;
    };
    auto add = [&](int field, int ix, int iz, double scale) {
        terms.push_back(SourceTerm{field, ix, iz});
        for (int it = 0; it < nt; ++it) amp.push_back(scale * sample(it));
    };
    if (wave == FD23_PSV) {
        double mxx = moment ? moment[0] : 0.0, mxz = moment ? moment[1] : 0.0,
               mzz = moment ? moment[2] : 0.0;
        if (kind == FD23_SRC_EXPLOSION) { mxx = 1.0; mxz = 0.0; mzz = 1.0; }
        if (kind == FD23_SRC_MOMENT_P) {
            const double g = f * dt / h;
            add(FD23_TXX, xs, zs, -(mxx * g));
            add(FD23_TXX, xs - 1, zs, mxx * g);
            add(FD23_TZZ, xs, zs, -(mzz * g));
            add(FD23_TZZ, xs - 1, zs, mzz * g);
            for (int x = xs - 1; x <= xs; ++x)
                for (int z = zs; z <= zs + 1; ++z) {
                    add(FD23_TXZ, x, z, -(mxz * g * 0.25));
                    add(FD23_TXZ, x - 1, z, mxz * g * 0.25);
                }
        } else {
            add(FD23_TXX, xs, zs, -(mxx * f));
            add(FD23_TZZ, xs, zs, -(mzz * f));
            if (kind != FD23_SRC_EXPLOSION || mxz != 0.0)
                for (int x = xs - 1; x <= xs; ++x)
                    for (int z = zs; z <= zs + 1; ++z) add(FD23_TXZ, x, z, -(mxz * f * 0.25));
        }
    } else {
        const double mxy = moment ? moment[0] : 0.0, mzy = moment ? moment[1] : 0.0;
        if (kind == FD23_SRC_FORCE) {
            add(FD23_V, xs, zs, -(0.5 * mxy * f));
        } else if (kind == FD23_SRC_MOMENT_P) {
            const double g = f * dt / h;
            add(FD23_TX, xs, zs, -(0.5 * mxy * g));
            add(FD23_TX, xs - 1, zs, -(0.5 * mxy * g));
            add(FD23_TZ, xs, zs, -(0.5 * mzy * g));
            add(FD23_TZ, xs, zs + 1, -(0.5 * mzy * g));
            add(FD23_TX, xs - 1, zs, 0.5 * mxy * g);
            add(FD23_TX, xs - 2, zs, 0.5 * mxy * g);
            add(FD23_TZ, xs - 1, zs, 0.5 * mzy * g);
            add(FD23_TZ, xs - 1, zs + 1, 0.5 * mzy * g);
        } else {
            add(FD23_TX, xs, zs, -(0.5 * mxy * f));
            add(FD23_TX, xs - 1, zs, -(0.5 * mxy * f));
            add(FD23_TZ, xs, zs, -(0.5 * mzy * f));
            add(FD23_TZ, xs, zs + 1, -(0.5 * mzy * f));
        }
    }
}

// ---------------------------------------------------------------------------
// Hybrid box, host side.

// Incident field on the ring cells of a bx x bz box from two displacement
// planes of (bx+8) x (bz+8) values (box cell (i, j) at plane (i+4, j+4)):
// BOX::setboxsource, PD/box/box.cpp:120-196.  Velocities are the forward
// difference of the planes over dt; stresses come from the new planes with
// the box material, at the reference's reduced stencil order around the box
// centre, evaluated in the reference's expression order (FP64).
int box_incident_from_displacement(int bx, int bz, double dt, const double *bmat, const double *uo,
                                   const double *wo, const double *un, const double *wn, double *out)
{
    const int nring = box_nsub(bx, bz) + box_nadd(bx, bz);
    const size_t nb = (size_t)bx * bz;
    const long pw = bx + 8;
    auto at = [pw](const double *a, int i, int j) { return a[i + (long)j * pw]; };
    // 4-term difference along (di, dj); `plus` selects the forward-staggered taps
    auto diff = [&](const double *a, int tx, int ty, int di, int dj, bool plus, const double *c) {
        const int p = plus ? 1 : 0;
        auto d = [&](int k) {
            return at(a, tx + (k + p) * di, ty + (k + p) * dj) - at(a, tx - (k + 1 - p) * di, ty - (k + 1 - p) * dj);
        };
        return c[0] * d(0) - c[1] * d(1) + c[2] * d(2) - c[3] * d(3);
    };
    for (int j = 0; j < bz; ++j)
        for (int i = 0; i < bx; ++i) {
            const int q = box_ring_index(i, j, bx, bz);
            if (q < 0) continue;
            const int tx = i + 4, ty = j + 4;
            const int oz = std::abs(ty - 3 - (bz + 1) / 2) - 1, ox = std::abs(tx - 3 - (bx + 1) / 2) - 1;
            const int ord = std::max(0, std::min(4, std::max(oz, ox)));
            const double *c = kCoef[ord];
            const double ux = diff(un, tx, ty, 1, 0, false, c), uz = diff(un, tx, ty, 0, 1, false, c);
            const double wx = diff(wn, tx, ty, 1, 0, true, c), wz = diff(wn, tx, ty, 0, 1, true, c);
            const size_t b = (size_t)j * bx + i;
            const double lam = bmat[b], mu = bmat[nb + b], mua = bmat[2 * nb + b];
            const double gam = lam + 2.0 * mu;
            out[q] = (at(un, tx, ty) - at(uo, tx, ty)) / dt;
            out[(size_t)nring + q] = (at(wn, tx, ty) - at(wo, tx, ty)) / dt;
            out[2 * (size_t)nring + q] = (gam * ux + lam * wz) / dt;
            out[3 * (size_t)nring + q] = (mua * (wx + uz)) / dt;
            out[4 * (size_t)nring + q] = (lam * ux + gam * wz) / dt;
        }
    return nring;
}

// Box material from the grid material (LAM MU MUA BU BW, dt/h scaled):
// MATERIAL::init_for_box_from_full, PD/material/material.cpp:39-97.  Box
// cells whose coefficients differ from the homogeneous source material by
// more than 1e-4 (relative) are overwritten in the grid material too.
int box_material(int nx, int nz, double *mat, int x0, int z0, int bx, int bz, double srcvp,
                 double srcvs, double srcden, double dt, double h, double *bmat)
{
    const size_t n = (size_t)nx * nz, nb = (size_t)bx * bz;
    const double mu0 = srcvs * srcvs * srcden;
    const double lam = (srcvp * srcvp * srcden - 2.0 * mu0) * dt / h;
    const double mu = mu0 * dt / h;
    const double b = 1.0 / srcden * dt / h;
    const double eps = 1e-4;
    int replaced = 0;
    for (int j = 0; j < bz; ++j)
        for (int i = 0; i < bx; ++i) {
            const size_t g = (size_t)(x0 + i) + (size_t)(z0 + j) * nx, k = (size_t)i + (size_t)j * bx;
            double &LAM = mat[g], &MU = mat[n + g], &MUA = mat[2 * n + g], &BU = mat[3 * n + g],
                   &BW = mat[4 * n + g];
            if (std::fabs(b - BU) > b * eps || std::fabs(b - BW) > b * eps || std::fabs(mu - MU) > mu * eps ||
                std::fabs(mu - MUA) > mu * eps || std::fabs(lam - LAM) > lam * eps) {
                BU = BW = b;
                MU = MUA = mu;
                LAM = lam;
                ++replaced;
            }
            bmat[k] = LAM;
            bmat[nb + k] = MU;
            bmat[2 * nb + k] = MUA;
            bmat[3 * nb + k] = BU;
            bmat[4 * nb + k] = BW;
        }
    return replaced;
}

}  // namespace fd23

namespace fd23 {

// CFL number of a model: max of vp (P-SV) or vs (SH) through cfl_number, as
// the builders above
double material_stab(int wave, const double *vp, const double *vs, size_t n, double h, double dt)
{
    const double *v = wave == FD23_PSV ? vp : vs;
    double vmax = -99999.0;
    for (size_t k = 0; k < n; ++k) vmax = std::max(vmax, v[k]);
    return cfl_number(vmax, h, dt);
}

}  // namespace fd23
