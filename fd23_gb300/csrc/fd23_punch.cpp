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

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "fd23_kernels.h"
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

// Work list of the phase holding step s->it: the 4-row blocks of the strips
// that touch a tile not steady at some step of the phase (or a source cell
// while the source runs), cut by the planner like a whole shot.  The sweep
// still narrows every item to the tiles live at its own step.
int phase_plan(fd23_solver *s, int *slot)
{
    const int P = s->punch_phase;
    const long long ph = s->it / P;
    const long long key = (s->punch_ver << 32) | ph;
    for (int k = 0; k < 3; ++k)
        if (s->phase[k].key == key) {
            *slot = k;
            return FD23_OK;
        }
    const int k = s->phase_next;
    s->phase_next = (k + 1) % 3;
    fd23_solver::PhasePlan &pp = s->phase[k];
    if (!pp.done) CK(cudaEventCreateWithFlags(&pp.done, cudaEventDisableTiming));
    else CK(cudaEventSynchronize(pp.done));  // its last launch has finished with the buffers
    const int t0 = (int)(ph * P), t1 = t0 + P;  // steps [t0, t1)
    const int nx = s->d.nx, nz = s->d.nz, nbx = s->punch_nbx, nbz = s->punch_nbz;
    std::vector<unsigned char> tile((size_t)nbx * nbz, 0);
    for (size_t t = 0; t < tile.size(); ++t) {
        const int2 w = s->h_punch[t];
        const long long lo = std::max<long long>((long long)w.x + 1, t0), hi = std::min<long long>(w.y, t1 - 1);
        tile[t] = (long long)w.y - w.x >= 2 && lo <= hi;
    }
    if (s->nterms > 0 && t0 <= s->tamp_nt)
        for (const int2 &c : s->h_tcell) tile[(size_t)(c.y / kPunchTZ) * nbx + c.x / kPunchTX] = 1;
    const int tx = fused_geom(s->d.wave, s->d.prec).tile_x, ntx = (nx + tx - 1) / tx, nzb = (nz + 3) / 4;
    std::vector<std::vector<unsigned char>> live(1, std::vector<unsigned char>((size_t)ntx * nzb, 0));
    for (int st = 0; st < ntx; ++st) {
        const int c0 = st * tx / kPunchTX, c1 = (std::min(st * tx + tx, nx) - 1) / kPunchTX;
        for (int zb = 0; zb < nzb; ++zb) {
            const int tz = std::min(4 * zb, nz - 1) / kPunchTZ;
            bool any = false;
            for (int c = c0; c <= c1 && !any; ++c) any = tile[(size_t)tz * nbx + c] != 0;
            live[0][(size_t)st * nzb + zb] = any;
        }
    }
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->d.device));
    TuneParams tp = s->tune;
    tp.per_sm = std::min(tp.per_sm, fused_per_sm(s->d.device, s->d.wave, s->d.prec));
    WorkPlan plan;
    const std::vector<ShotGeom> geo{ShotGeom{nx, nz, s->d.npml, s->d.topabsorb}};
    int rc = plan_work(geo, tx, sms, tp, plan, &live);
    if (rc) return rc;
    if (plan.nblocks == 0) {  // nothing live: one CTA without items (it still gathers the receivers)
        plan.off.assign(2, 0);
        plan.nblocks = 1;
    }
    auto grow = [](void **p, size_t *cap, size_t need) -> int {
        if (*cap >= need) return FD23_OK;
        cudaFree(*p);
        *p = nullptr;
        *cap = 0;
        const int r = dev_alloc(p, need);
        if (!r) *cap = need;
        return r;
    };
    const size_t ni = std::max<size_t>(1, plan.items.size()) * sizeof(WorkItem), no = plan.off.size() * sizeof(int);
    if ((rc = grow((void **)&pp.items, &pp.cap_items, ni)) || (rc = grow((void **)&pp.off, &pp.cap_off, no)))
        return rc;
    // through pinned memory, so the copies queue without waiting for the stream
    if (pp.cap_host < ni + no) {
        cudaFreeHost(pp.host);
        pp.host = nullptr;
        pp.cap_host = 0;
        CK(cudaMallocHost(&pp.host, ni + no));
        pp.cap_host = ni + no;
    }
    unsigned char *hb = (unsigned char *)pp.host;
    if (!plan.items.empty()) std::memcpy(hb, plan.items.data(), plan.items.size() * sizeof(WorkItem));
    std::memcpy(hb + ni, plan.off.data(), no);
    if (!plan.items.empty())
        CK(cudaMemcpyAsync(pp.items, hb, plan.items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(pp.off, hb + ni, no, cudaMemcpyHostToDevice, s->stream));
    pp.nblocks = plan.nblocks;
    pp.key = key;
    *slot = k;
    return FD23_OK;
}

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

int fd23_set_punch_phase(fd23_solver *s, int steps)
{
    if (!s || steps < 0) return FD23_ERR_ARG;
    s->punch_phase = steps;
    ++s->punch_ver;
    return FD23_OK;
}

int fd23_set_punch(fd23_solver *s, const int *first, const int *last, int nbx, int nbz)
{
    if (!s) return FD23_ERR_ARG;
    CK(cudaSetDevice(s->d.device));
    CK(cudaStreamSynchronize(s->stream));
    ++s->punch_ver;
    if (!first && !last) {  // windows off
        cudaFree(s->d_punch);
        s->d_punch = nullptr;
        s->punch_nbx = s->punch_nbz = 0;
        s->h_punch.clear();
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
    s->h_punch = w;
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
