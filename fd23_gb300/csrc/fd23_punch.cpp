// usepunch: step windows of 32 x 16 tiles (host side).
//
// The reference (PD/slide/cu_slide.cu:6-66, PN/slide/cu_slide.cu, SH/slide/
// cu_slide.cu) reads a travel-time file of nx*nz values (row-major, rows of
// nx), takes the smallest and the largest time of every 32 x 16 tile and
// turns them into the steps
//     first = int((tmin - before) / dt),   last = int((tmax + after) / dt);
// its sweep kernels update the cells of a tile at step it only while
// first < it < last (PD/fd/cu_fd.cu:16-23).  PD reads doubles and computes in
// double; PN and SH read floats and compute in float.  Both forms are here
// (elem_bytes 8 or 4).  Extensions: grids that are not whole tiles (the
// reference requires nx % 32 == 0 and nz % 16 == 0) get partial edge tiles;
// the float-to-int conversion saturates (NaN gives 0) where the reference's
// is undefined.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdio>
#include <vector>

#include "fd23_solver.h"

namespace fd23 {

namespace {

template <class T>
int to_step(T v)
{
    if (v != v) return 0;
    if (v >= (T)2147483647.0) return INT_MAX;
    if (v <= (T)-2147483648.0) return INT_MIN;
    return (int)v;  // truncation toward zero, as int() in the reference
}

template <class T>
void windows(const T *t, int nx, int nz, T before, T after, T dt, int *first, int *last)
{
    const int nbx = (nx + kPunchTX - 1) / kPunchTX, nbz = (nz + kPunchTZ - 1) / kPunchTZ;
    for (int bz = 0; bz < nbz; ++bz)
        for (int bx = 0; bx < nbx; ++bx) {
            T lo = (T)1e28, hi = (T)-1e28;
            for (int j = bz * kPunchTZ; j < std::min(nz, (bz + 1) * kPunchTZ); ++j)
                for (int i = bx * kPunchTX; i < std::min(nx, (bx + 1) * kPunchTX); ++i) {
                    const T v = t[(size_t)j * nx + i];
                    lo = std::fmin(lo, v);
                    hi = std::fmax(hi, v);
                }
            first[bz * nbx + bx] = to_step<T>((lo - before) / dt);
            last[bz * nbx + bx] = to_step<T>((hi + after) / dt);
        }
}

}  // namespace

int mirror_sets(fd23_solver *s, cudaStream_t st)
{
    if (!s->fused) return FD23_OK;  // the two-pass sweep keeps one set
    const int a = s->par, b = 1 - a;
    for (int f = 0; f < s->nfld; ++f)
        CK(cudaMemcpyAsync(s->fld[b][f], s->fld[a][f], s->L.elems() * s->es, cudaMemcpyDeviceToDevice, st));
    for (int p = 0; p < s->npsi; ++p)
        if (s->psi_elems[p])
            CK(cudaMemcpyAsync(s->psi[b][p], s->psi[a][p], s->psi_elems[p] * s->cs, cudaMemcpyDeviceToDevice,
                               st));
    return FD23_OK;
}

}  // namespace fd23

using namespace fd23;

extern "C" {

int fd23_punch_tiles(int nx, int nz, int *nbx, int *nbz)
{
    if (nx <= 0 || nz <= 0 || !nbx || !nbz) return FD23_ERR_ARG;
    *nbx = (nx + kPunchTX - 1) / kPunchTX;
    *nbz = (nz + kPunchTZ - 1) / kPunchTZ;
    return FD23_OK;
}

int fd23_punch_windows(const void *times, int elem_bytes, int nx, int nz, double before, double after,
                       double dt, int *first, int *last)
{
    if (!times || nx <= 0 || nz <= 0 || !first || !last || !(dt != 0.0)) return FD23_ERR_ARG;
    if (elem_bytes == 8)
        windows<double>((const double *)times, nx, nz, before, after, dt, first, last);
    else if (elem_bytes == 4)
        windows<float>((const float *)times, nx, nz, (float)before, (float)after, (float)dt, first, last);
    else
        return FD23_ERR_ARG;
    return FD23_OK;
}

int fd23_read_punch(const char *timefile, int elem_bytes, int nx, int nz, double before, double after, double dt,
                    int *first, int *last)
{
    if (!timefile || (elem_bytes != 4 && elem_bytes != 8) || nx <= 0 || nz <= 0) return FD23_ERR_ARG;
    std::FILE *fp = std::fopen(timefile, "rb");
    if (!fp) return FD23_ERR_ARG;
    const size_t n = (size_t)nx * nz;
    std::vector<unsigned char> buf(n * elem_bytes);
    const size_t got = std::fread(buf.data(), 1, buf.size(), fp);
    std::fclose(fp);
    if (got != buf.size()) return FD23_ERR_ARG;  // missing or short file
    return fd23_punch_windows(buf.data(), elem_bytes, nx, nz, before, after, dt, first, last);
}

int fd23_set_punch(fd23_solver *s, const int *first, const int *last, int nbx, int nbz)
{
    if (!s) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    CK(cudaStreamSynchronize(s->stream));
    if (!first && !last) {  // windows off
        cudaFree(s->d_punch);
        s->d_punch = nullptr;
        s->punch_nbx = s->punch_nbz = 0;
        return FD23_OK;
    }
    int wx = 0, wz = 0;
    fd23_punch_tiles(s->d.nx, s->d.nz, &wx, &wz);
    if (!first || !last || nbx != wx || nbz != wz) return FD23_ERR_ARG;
    if (s->box_on) return FD23_ERR_UNSUPPORTED;
    const size_t n = (size_t)nbx * nbz;
    std::vector<int2> w(n);
    for (size_t k = 0; k < n; ++k) w[k] = make_int2(first[k], last[k]);
    if (!s->d_punch) {
        const int rc = dev_alloc((void **)&s->d_punch, n * sizeof(int2));
        if (rc) return rc;
    }
    CK(cudaMemcpy(s->d_punch, w.data(), n * sizeof(int2), cudaMemcpyHostToDevice));
    s->punch_nbx = nbx;
    s->punch_nbz = nbz;
    // tiles left alone at two steps in a row are skipped by the fused sweep,
    // which needs both buffer sets to agree on them from here on
    const int rc = mirror_sets(s, s->stream);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream));
    return FD23_OK;
}

}  // extern "C"
