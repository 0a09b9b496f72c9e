// Work plans of the fused sweep (host side).
//
// A shot is cut into strips of tile_x output columns and 4-row blocks.  Every
// block gets an estimated cost (blocks that touch the CPML run the general
// per-cell path and cost more: wx for the x-CPML, wz for the z-CPML and the
// edge rows).  CTAs are shared out between shots in proportion to their cost,
// then every shot's blocks are cut, strip-major, into contiguous ranges of
// equal cost; a range that crosses strips becomes several items.  A CTA never
// mixes shots, so it keeps one shot descriptor.
#include <algorithm>
#include <cmath>

#include "fd23_internal.h"

namespace fd23 {

namespace {

// cost of block (strip, zb) of a shot
double block_cost(const ShotGeom &g, int tile_x, int strip, int zb, const TuneParams &tp)
{
    const int x0 = strip * tile_x;
    const bool xp = (x0 - 4 < std::max(g.npml, 4)) || (x0 + tile_x + 4 > std::min(g.nx - g.npml, g.nx - 4));
    const int r0 = 4 * zb, r1 = r0 + 3;
    const bool zp = (r1 >= std::min(g.nz - g.npml, g.nz - 4)) || r0 < 4 || (g.topabsorb && r0 < g.npml);
    return xp ? tp.wx : (zp ? tp.wz : 1.0);
}

}  // namespace

int plan_work(const std::vector<ShotGeom> &shots, int tile_x, int sms, const TuneParams &tp, WorkPlan &plan)
{
    const int ns = (int)shots.size();
    if (ns <= 0 || tile_x <= 0 || sms <= 0) return FD23_ERR_ARG;
    std::vector<std::vector<double>> cum(ns);
    std::vector<int> ntx(ns), nzb(ns), nmin(ns);
    double total = 0.0;
    for (int k = 0; k < ns; ++k) {
        const ShotGeom &g = shots[k];
        ntx[k] = (g.nx + tile_x - 1) / tile_x;
        nzb[k] = (g.nz + 3) / 4;
        const long long nb = (long long)ntx[k] * nzb[k];
        cum[k].assign((size_t)nb + 1, 0.0);
        for (long long b = 0; b < nb; ++b)
            cum[k][b + 1] = cum[k][b] + block_cost(g, tile_x, (int)(b / nzb[k]), (int)(b % nzb[k]), tp);
        total += cum[k][nb];
        nmin[k] = std::max(1, (ntx[k] + 1) / 2);  // keeps every CTA within 4 items
    }
    // CTAs: the resident slots times the oversubscription, shared by cost
    const long long slots = std::max(1LL, (long long)std::llround(sms * tp.per_sm * std::max(tp.oversub, 0.05)));
    std::vector<int> nc(ns);
    for (int k = 0; k < ns; ++k) {
        const long long nb = (long long)ntx[k] * nzb[k];
        const double share = slots * cum[k][nb] / total;
        nc[k] = (int)std::min<long long>(nb, std::max<long long>(nmin[k], std::llround(share)));
    }
    plan.items.clear();
    plan.off.assign(1, 0);
    plan.cta0.assign(ns, 0);
    plan.ncta.assign(ns, 0);
    for (int k = 0; k < ns; ++k) {
        const long long nb = (long long)ntx[k] * nzb[k];
        const int n = nc[k];
        const std::vector<double> &c = cum[k];
        plan.cta0[k] = (int)plan.off.size() - 1;
        plan.ncta[k] = n;
        long long b0 = 0;
        for (int q = 0; q < n; ++q) {
            long long b1;
            if (q == n - 1) {
                b1 = nb;
            } else {
                const double target = c[nb] * (double)(q + 1) / (double)n;
                b1 = std::lower_bound(c.begin() + b0 + 1, c.end(), target) - c.begin();
                b1 = std::max(b1, b0 + 1);
                b1 = std::min(b1, nb - (n - 1 - q));  // leave a block for every later CTA
            }
            while (b0 < b1) {
                const int strip = (int)(b0 / nzb[k]);
                const long long send = (long long)(strip + 1) * nzb[k];
                const long long e = std::min(b1, send);
                plan.items.push_back(WorkItem{k, strip * tile_x, (int)(b0 - (long long)strip * nzb[k]) * 4,
                                              (int)(e - (long long)strip * nzb[k]) * 4});
                b0 = e;
            }
            plan.off.push_back((int)plan.items.size());
        }
    }
    plan.nblocks = (int)plan.off.size() - 1;
    for (int c = 0; c < plan.nblocks; ++c)
        if (plan.off[c + 1] - plan.off[c] > 4) return FD23_ERR_ARG;
    return FD23_OK;
}

}  // namespace fd23
