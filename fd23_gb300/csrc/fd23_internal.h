// Internal declarations shared by the host C++ and the CUDA translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <vector_types.h>

#include "../../include/fd23.h"

namespace fd23 {

extern const double kCoef[5][4];

// ---------------------------------------------------------------------------
// HBM layout of one wavefield / material array.
//
// Every 2-D array is stored with zero padding around the physical grid so
// that the stencil halo (4 cells) and every row segment a thread block copies
// is in bounds and 16-byte aligned, and so that cells outside the grid read
// as zero (the reference's zero halo, PD/fd/cu_fd.cu:70-89) without any
// bounds test in the sweep.  Element (ix, iz) lives at
//     origin + iz*pitch + ix,   origin = kZPad*pitch + kXPad
// with pitch a multiple of 32 elements.  The padding is written once (zero)
// and never again: kernels store only cells inside the grid.
constexpr int kXPad = 8;
constexpr int kZPad = 8;

struct Layout {
    int nx = 0, nz = 0;
    int pitch = 0;        // elements per stored row
    int rows = 0;         // stored rows (padding included)
    long long origin = 0; // element offset of (0, 0)
    size_t elems() const { return (size_t)pitch * (size_t)rows; }
};

// x extent covered by the sweep tiles may overhang the grid; the layout is
// sized for `cover_x` columns and `cover_z` rows plus halo padding.
Layout make_layout(int nx, int nz, int cover_x, int cover_z);

struct SourceTerm {
    int field, ix, iz;
};

// ---------------------------------------------------------------------------
// Device-side description of one shot.  S = storage type of wavefields and
// material, C = arithmetic type (also the type of memory variables, CPML
// coefficients, source amplitudes and seismograms).
template <class S, class C>
struct Shot {
    S *f[2][5];         // ping-pong wavefields (P-SV: U W Txx Txz Tzz; SH: V Tx Tz)
    const S *mat[5];    // P-SV: LAM MU MUA BU BW; SH: MUX MUZ BV
    C *psi[2][8];       // ping-pong memory variables, reference index maps
    const C *cpml;      // b | c | k blocks, reference component order
    int nx, nz, npml, topabsorb;
    int pitch;
    long long origin;
    int cpml_blk;       // elements per b / c / k block
    // point source
    int nterms;
    const int4 *terms;  // (field, ix, iz, 0)
    const C *tamp;      // [nterms][tamp_nt]
    int tamp_nt;
    // receivers: padded element offsets, seismograms [record][n]
    int nrec[2];
    const long long *rec[2];
    C *seis[2];
};

// Work list entry of the fused sweep: one x-strip of one shot, rows [z0, z1)
struct WorkItem {
    int shot, x0, z0, z1;
};

// host builders (fd23_host.cpp)
int build_psv_material(int nx, int nz, double h, double dt, const double *vp, const double *vs,
                       const double *den, double *out, double *stab);
int build_sh_material(int nx, int nz, double h, double dt, const double *vs, const double *den,
                      double *out, double *stab);
void build_cpml_profile(int npml, double start, int n, double pml_dt, double pml_r, double pml_v,
                        double pml_fc, double *b, double *c, double *k);
void build_cpml(int wave, int nx, int nz, int npml, double pml_dt, double pml_r, double pml_v,
                double pml_fc, std::vector<double> &bck);
void moment_psv(double strike, double dip, double rake, double azimuth, double m[3]);
void moment_sh(double strike, double dip, double rake, double azimuth, double m[2]);
int wavelet_gaussian(double dt, int alpha, double *out, int cap);
int wavelet_trapezoid(double dt, double t1, double t2, double t3, double *out, int cap);
int wavelet_ricker(double dt, double f0, double t0, double *out, int cap);
void build_source_terms(int wave, int kind, int xs, int zs, const double *moment, double h,
                        double dt, const double *src, int lsrc, int nt,
                        std::vector<SourceTerm> &terms, std::vector<double> &amp);

}  // namespace fd23
