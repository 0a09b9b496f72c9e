// Internal declarations shared by the host C++ and the CUDA translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <vector_types.h>

#include "../../include/fd23.h"

#if defined(__CUDACC__)
#define FD23_HD __host__ __device__
#else
#define FD23_HD
#endif

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
// Hybrid box (P-SV).  A box is the grid cells [x0, x0+bx) x [z0, z0+bz),
// bx, bz >= 16.  Its two rings, box-local (PD/box/box.cpp:59-95 for a square
// box around the source, generalised to any rectangle):
//   sub ring: the cells within 4 of the box edge;
//   add ring: the cells within 4 of the edge of [4, bx-4) x [4, bz-4).
// The incident field of one step is stored on the ring cells, [5][nring]:
// sub-ring cells first, then add-ring cells, each ring row by row.
constexpr int kBoxMin = 16;

FD23_HD inline int box_nsub(int bx, int bz) { return 8 * (bx + bz - 8); }
FD23_HD inline int box_nadd(int bx, int bz) { return 8 * (bx + bz - 24); }

// row-major position of cell (i, j) of a 4-wide band along the edge of a
// w x h rectangle (w, h >= 8); the cell must lie in the band
FD23_HD inline int band_index(int i, int j, int w, int h)
{
    if (j < 4) return j * w + i;
    if (j >= h - 4) return 4 * w + (h - 8) * 8 + (j - (h - 4)) * w + i;
    return 4 * w + (j - 4) * 8 + (i < 4 ? i : i - (w - 8));
}
// ring position of box cell (bi, bj): [0, nsub) sub ring, [nsub, nring) add
// ring, -1 for cells in neither ring (or outside the box)
FD23_HD inline int box_ring_index(int bi, int bj, int bx, int bz)
{
    if (bi < 0 || bj < 0 || bi >= bx || bj >= bz) return -1;
    if (bi < 4 || bi >= bx - 4 || bj < 4 || bj >= bz - 4) return band_index(bi, bj, bx, bz);
    const int ai = bi - 4, aj = bj - 4, w = bx - 8, h = bz - 8;
    if (ai < 4 || ai >= w - 4 || aj < 4 || aj >= h - 4) return box_nsub(bx, bz) + band_index(ai, aj, w, h);
    return -1;
}

// TMA tensor maps of one shot (opaque 128-byte CUtensorMap objects built on
// the host by cuTensorMapEncodeTiled).  Each is a 3-D view [field][row]
// [column] of a contiguous block of padded arrays (the wavefields of one
// buffer set, or the materials), one map per copy shape of the fused sweep.
struct alignas(128) TmaDesc {
    unsigned char bytes[128];
};
struct ShotMaps {
    TmaDesc uw[2];  // stencil inputs of buffer set 0 / 1 (P-SV U W, SH V), box UWW x 4 x NV
    TmaDesc t[2];   // old stresses of buffer set 0 / 1, box PWW x 4 x NT
    TmaDesc ms;     // stress-update material, box PWW x 4 x NMS
    TmaDesc mv;     // velocity-update material, box PWW x 4 x NMV
    TmaDesc idx;    // material-table indices (bytes), 2-D [row][column], box kIdxBoxW x 8
};

// Tensor maps of the two-step sweep (fd23_fused2.cu): the same 3-D views with
// its wider boxes (input rows of 264 columns, point-wise rows of 256).
struct ShotMaps2 {
    TmaDesc uw[2];  // U W of buffer set 0 / 1, box 264 x 4 x 2
    TmaDesc t[2];   // stresses of buffer set 0 / 1, box 256 x 4 x 3
    TmaDesc ms;     // stress-update material, box (256 or 264) x 4 x 3
    TmaDesc mv;     // velocity-update material, box (256 or 264) x 4 x 2
};

// Material table (mktable, PD/material/mktable.cpp): every cell's material
// tuple (P-SV LAM MU MUA BU BW, SH MUX MUZ BV, storage values) as a one-byte
// index into a table of at most kTabEntries tuples; entry 0 is the zero tuple
// of the padding.  The fused sweep copies 8 index rows of kIdxBoxW bytes per
// iteration (16-byte aligned start, so wider than the point-wise rows).
constexpr int kTabEntries = 256;
constexpr int kIdxBoxW = 160;

// Device view of the box of one shot: residual field r and box material,
// bx*bz each, row-major; `inc` = the incident field of the current step.
template <class C>
struct Box {
    int on;
    int x0, z0, bx, bz;
    int nsub, nring;
    C *r[5];            // U W Txx Txz Tzz
    const C *rmat[5];   // LAM MU MUA BU BW (dt/h scaled)
    const C *inc;       // [5][nring]
    const int2 *cells;  // ring position -> box-local (bi, bj)
};

// Step windows of the tiles of a shot (usepunch, PD/fd/cu_fd.cu:16-23,
// PD/slide/cu_slide.cu): the cells of tile (ix / kPunchTX, iz / kPunchTZ)
// are updated at step it only while first < it < last; outside that window
// their stresses, velocities and memory variables keep their values.
constexpr int kPunchTX = 32, kPunchTZ = 16;
struct Punch {
    const int2 *win;  // [nbz][nbx] (first, last); null: every cell is updated
    int nbx, nbz;
};
FD23_HD inline bool punch_active(const Punch &p, int ix, int iz, int it)
{
    if (!p.win) return true;
    const int2 w = p.win[(iz / kPunchTZ) * p.nbx + ix / kPunchTX];
    return w.x < it && it < w.y;
}
// A tile whose cells were left alone at step it-1 and are left alone at
// step it holds the same values in both ping-pong buffer sets, so the fused
// sweep may skip it at step it.
FD23_HD inline bool punch_steady(int2 w, int it)
{
    return !(w.x < it && it <= w.y && (long long)w.y - w.x >= 2);
}

// ---------------------------------------------------------------------------
// Device-side description of one shot.  S = storage type of wavefields and
// material, C = arithmetic type (also the type of memory variables, CPML
// coefficients, source amplitudes and seismograms).
template <class S, class C>
struct alignas(16) Shot {
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
    // receivers of each wavefield: padded element offsets, seismograms [record][n]
    int nrec[5];
    const long long *rec[5];
    C *seis[5];
    const ShotMaps *maps;  // tensor maps of the fused sweep's copies (device memory)
    int cta0, ncta;     // CTAs of the launch working on this shot (receiver gather split)
    Punch punch;        // tile step windows (punch.win == nullptr: none)
    const unsigned char *midx;  // material-table indices, padded layout (nullptr: no table)
    const S *mtab;              // table [material array][kTabEntries], storage values
    // two-step sweep only: its tensor maps, the memory variables of the
    // step in between (written and read within one launch), and the
    // receivers each work item records at that step: entries (field, ix, iz,
    // receiver) sorted by iz, velocity entries of item k in
    // [rec2_off[2k], rec2_off[2k+1]), stress entries up to rec2_off[2k+2]
    const ShotMaps2 *maps2;
    const void *mat16[5];  // FP16 copies of the material (null: the sweep reads `mat`)
    C *psim[8];
    const int4 *rec2;
    const int *rec2_off;
    Box<C> box;         // hybrid box (box.on == 0: none); single shots only
    // (the batched sweep copies and reads the fields before maps2 only)
};

// Work list entry of the fused sweep: one x-strip of one shot, rows [z0, z1)
struct WorkItem {
    int shot, x0, z0, z1;
};

// Work plan of one fused launch over one or more shots: CTA c works on
// items[off[c] .. off[c+1]) (at most 4, all of one shot); shot k is worked
// on by CTAs [cta0[k], cta0[k] + ncta[k]).
struct ShotGeom {
    int nx, nz, npml, topabsorb;
    int xoff = 0;  // first strip's first column (plan_work sets it: a multiple of 8 in (-tile_x, 0])
};
struct TuneParams {
    double wx = 4.0, wz = 3.0;  // relative cost of 4-row blocks touching the x / z CPML
    int per_sm = 3;             // CTAs resident per SM the plan is sized for
    double oversub = 1.0;       // CTAs launched per resident slot
    int bands = 1;              // cut every strip on its own (plan_work)
    int shift = 1;              // let plan_work move the strips' origin left of column 0
    int fast = 0;               // single-shot FP32: the sweep with uniform fast iterations
};
struct WorkPlan {
    std::vector<WorkItem> items;
    std::vector<int> off, cta0, ncta;
    int nblocks = 0;
};
// live (optional): per shot, per 4-row block (strip-major, strip * nzb + zb)
// whether it is planned at all; without it every block is
int plan_work(const std::vector<ShotGeom> &shots, int tile_x, int sms, const TuneParams &tp,
              WorkPlan &plan, const std::vector<std::vector<unsigned char>> *live = nullptr);

// host builders (fd23_host.cpp)
int build_psv_material(int nx, int nz, double h, double dt, const double *vp, const double *vs,
                       const double *den, double *out, double *stab);
int build_sh_material(int nx, int nz, double h, double dt, const double *vs, const double *den,
                      double *out, double *stab);
void build_cpml_profile(int npml, double start, int n, double pml_dt, double pml_r, double pml_v,
                        double pml_fc, double *b, double *c, double *k);
void build_cpml(int wave, int nx, int nz, int npml, double pml_dt, double pml_r, double pml_v,
                double pml_fc, std::vector<double> &bck);
double material_stab(int wave, const double *vp, const double *vs, size_t n, double h, double dt);
void moment_psv(double strike, double dip, double rake, double azimuth, double m[3]);
void moment_sh(double strike, double dip, double rake, double azimuth, double m[2]);
int wavelet_gaussian(double dt, int alpha, double *out, int cap);
int wavelet_trapezoid(double dt, double t1, double t2, double t3, double *out, int cap);
int wavelet_ricker(double dt, double f0, double t0, double *out, int cap);
void build_source_terms(int wave, int kind, int xs, int zs, const double *moment, double h,
                        double dt, const double *src, int lsrc, int nt,
                        std::vector<SourceTerm> &terms, std::vector<double> &amp);

// hybrid-box host builders (fd23_host.cpp)
int box_incident_from_displacement(int bx, int bz, double dt, const double *bmat, const double *uo,
                                   const double *wo, const double *un, const double *wn, double *out);
int box_material(int nx, int nz, double *mat, int x0, int z0, int bx, int bz, double srcvp,
                 double srcvs, double srcden, double dt, double h, double *bmat);

}  // namespace fd23
