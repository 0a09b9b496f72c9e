// Work plans of the fused sweep (host side).
//
// A shot is cut into strips of tile_x output columns (from an origin at or
// left of column 0, best_xoff) and 4-row blocks.  Every
// block gets an estimated cost (blocks that touch the CPML run the general
// per-cell path and cost more: wx for the x-CPML, wz for the z-CPML and the
// edge rows).  CTAs are shared out between shots in proportion to their cost,
// then every shot's blocks are cut, strip-major, into contiguous ranges of
// equal cost; a range that crosses strips becomes several items.  A CTA never
// mixes shots, so it keeps one shot descriptor.  With a live mask only the
// live blocks are planned (runs of consecutive live blocks of a strip take
// the place of strips).
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "fd23_internal.h"

namespace fd23 {

namespace {

// strip `strip` of a shot runs the CPML / reduced-order path in its x range
// (its 4-column stress halos included)
bool strip_xp(const ShotGeom &g, int tile_x, int strip)
{
    const int x0 = g.xoff + strip * tile_x;
    return (x0 - 4 < std::max(g.npml, 4)) || (x0 + tile_x + 4 > std::min(g.nx - g.npml, g.nx - 4));
}

// cost of block row zb of a strip clear of the x-CPML
double row_cost(const ShotGeom &g, int zb, const TuneParams &tp)
{
    const int r0 = 4 * zb, r1 = r0 + 3;
    const bool zp = (r1 >= std::min(g.nz - g.npml, g.nz - 4)) || r0 < 4 || (g.topabsorb && r0 < g.npml);
    return zp ? tp.wz : 1.0;
}

// cost of block (strip, zb) of a shot
double block_cost(const ShotGeom &g, int tile_x, int strip, int zb, const TuneParams &tp)
{
    return strip_xp(g, tile_x, strip) ? tp.wx : row_cost(g, zb, tp);
}

int strips_of(const ShotGeom &g, int tile_x) { return (g.nx - g.xoff + tile_x - 1) / tile_x; }

// Strip origin of a shot: the multiple of 8 in (-tile_x, 0] whose strips
// cost least in total (ties: the one nearest 0).  Moving the origin left
// can put both x-CPML zones and their 4-column halos into fewer strips: on
// the 4000-column grid with a 40-cell CPML, origin 0 makes three strips run
// the CPML path (0, 32 and 33, strip 32 through its halo only), origin -8
// (the first that does) two.  Copies that start left of column -8 read
// zeros, as the padding columns hold.
int best_xoff(ShotGeom g, int tile_x, const TuneParams &tp)
{
    const int nzb = (g.nz + 3) / 4;
    double interior = 0.0;
    for (int zb = 0; zb < nzb; ++zb) interior += row_cost(g, zb, tp);
    int best = 0;
    double best_cost = 0.0;
    for (int xo = 0; xo > -tile_x; xo -= 8) {
        g.xoff = xo;
        double cost = 0.0;
        const int ntx = strips_of(g, tile_x);
        for (int s = 0; s < ntx; ++s) cost += strip_xp(g, tile_x, s) ? tp.wx * nzb : interior;
        if (xo == 0 || cost < best_cost - 1e-9) {
            best = xo;
            best_cost = cost;
        }
    }
    return best;
}

// Banded cut of one shot (every block planned) for n CTAs: every strip is
// cut on its own into ranges of equal cost, each strip getting the fewest
// CTAs that keep its ranges at or below the largest per-CTA cost of the best
// split (CTAs handed out one at a time to the strip with the costliest
// ranges).  Strips of the same cost profile (all the interior strips) get the
// same row boundaries, so neighbouring strips sweep the same rows at the same
// time and the columns their copies share are still in L2 for the second
// reader.  False (nothing added) when there are fewer CTAs than strips.
bool cut_bands(const std::vector<double> &c, int shot, int xoff, int ntx, int nzb, int tile_x, int n, WorkPlan &plan)
{
    if (n < ntx) return false;
    std::vector<double> cost(ntx);
    for (int s = 0; s < ntx; ++s) cost[s] = c[(size_t)(s + 1) * nzb] - c[(size_t)s * nzb];
    std::vector<int> ns(ntx, 1);
    for (int left = n - ntx; left > 0; --left) {
        int w = -1;
        for (int s = 0; s < ntx; ++s)
            if (ns[s] < nzb && (w < 0 || cost[s] * ns[w] > cost[w] * ns[s])) w = s;
        if (w < 0) break;
        ++ns[w];
    }
    double m = 0.0;
    for (int s = 0; s < ntx; ++s) m = std::max(m, cost[s] / ns[s]);
    for (int s = 0; s < ntx; ++s) {
        int k = 1;
        while (k < ns[s] && cost[s] / k > m * (1.0 + 1e-12)) ++k;
        ns[s] = k;
    }
    for (int s = 0; s < ntx; ++s) {
        const size_t a = (size_t)s * nzb;
        long long b0 = 0;
        for (int q = 0; q < ns[s]; ++q) {
            long long b1 = nzb;
            if (q < ns[s] - 1) {
                const double target = c[a] + cost[s] * (double)(q + 1) / (double)ns[s];
                b1 = (long long)(std::lower_bound(c.begin() + a + b0 + 1, c.begin() + a + nzb, target) - (c.begin() + a));
                b1 = std::max(b1, b0 + 1);
                b1 = std::min(b1, (long long)nzb - (ns[s] - 1 - q));
            }
            plan.items.push_back(WorkItem{shot, xoff + s * tile_x, (int)b0 * 4, (int)b1 * 4});
            plan.off.push_back((int)plan.items.size());
            b0 = b1;
        }
    }
    return true;
}

}  // namespace

// Cuts the nb planned blocks of one shot (cumulative costs c; run_begin[r]
// = first block of run r, a run being consecutive blocks of one strip) into
// n contiguous ranges of near-equal cost, none touching more than 4 runs;
// false if the last range would need more.
bool cut_shot(const std::vector<double> &c, long long nb, const std::vector<long long> &run_of,
              const std::vector<long long> &run_begin, int n, std::vector<long long> &ends)
{
    ends.clear();
    long long b0 = 0;
    for (int q = 0; q < n; ++q) {
        const long long r4 = run_of[b0] + 4;
        const long long cap = r4 < (long long)run_begin.size() ? run_begin[r4] : nb;  // at most 4 runs
        long long b1;
        if (q == n - 1) {
            b1 = nb;
            if (b1 > cap) return false;
        } else {
            const double target = c[nb] * (double)(q + 1) / (double)n;
            b1 = std::lower_bound(c.begin() + b0 + 1, c.end(), target) - c.begin();
            b1 = std::max(b1, b0 + 1);
            b1 = std::min(b1, nb - (n - 1 - q));  // leave a block for every later CTA
            b1 = std::min(b1, cap);
        }
        ends.push_back(b1);
        b0 = b1;
    }
    return true;
}

int plan_work(const std::vector<ShotGeom> &shots, int tile_x, int sms, const TuneParams &tp, WorkPlan &plan,
              const std::vector<std::vector<unsigned char>> *live)
{
    const int ns = (int)shots.size();
    if (ns <= 0 || tile_x <= 0 || sms <= 0) return FD23_ERR_ARG;
    if (live && (int)live->size() != ns) return FD23_ERR_ARG;
    // planned blocks of every shot (all of them, or the live ones), strip-major,
    // with their runs and cumulative costs
    std::vector<std::vector<long long>> blk(ns), run_of(ns), run_begin(ns);
    std::vector<std::vector<double>> cum(ns);
    std::vector<int> nzb(ns), nmin(ns);
    std::vector<long long> nbk(ns);
    double total = 0.0;
    long long sum_min = 0;
    // strip origins: planned over every block, the cheapest; with a live mask
    // (laid out over strips from column 0) at column 0
    // (FD23_STRIP_SHIFT=0 in the environment keeps every origin at column 0)
    static const bool no_shift = [] {
        const char *v = std::getenv("FD23_STRIP_SHIFT");
        return v && std::atoi(v) == 0;
    }();
    std::vector<ShotGeom> geo(shots);
    for (auto &g : geo) g.xoff = (!live && tp.shift && !no_shift) ? best_xoff(g, tile_x, tp) : 0;
    for (int k = 0; k < ns; ++k) {
        const ShotGeom &g = geo[k];
        const int ntx = strips_of(g, tile_x);
        nzb[k] = (g.nz + 3) / 4;
        const long long all = (long long)ntx * nzb[k];
        if (live && (long long)(*live)[k].size() != all) return FD23_ERR_ARG;
        cum[k].assign(1, 0.0);
        long long prev = -2;
        for (long long b = 0; b < all; ++b) {
            if (live && !(*live)[k][b]) continue;
            if (b != prev + 1 || b % nzb[k] == 0) run_begin[k].push_back((long long)blk[k].size());
            run_of[k].push_back((long long)run_begin[k].size() - 1);
            blk[k].push_back(b);
            cum[k].push_back(cum[k].back() + block_cost(g, tile_x, (int)(b / nzb[k]), (int)(b % nzb[k]), tp));
            prev = b;
        }
        nbk[k] = (long long)blk[k].size();
        total += cum[k].back();
        const long long runs = (long long)run_begin[k].size();
        nmin[k] = (int)std::min<long long>(nbk[k], std::max(1LL, (runs + 1) / 2));  // within 4 items
        sum_min += nmin[k];
    }
    // CTA count: the resident slots times the oversubscription, rounded up to
    // whole waves once the per-shot minimums are met
    const long long slots = std::max(1LL, (long long)sms * std::max(1, tp.per_sm));
    long long want = std::max(1LL, (long long)std::llround(slots * std::max(tp.oversub, 0.05)));
    want = std::max(want, sum_min);
    if (want > slots) want = (want + slots - 1) / slots * slots;
    long long cap_all = 0;
    for (int k = 0; k < ns; ++k) cap_all += nbk[k];
    want = std::min(want, cap_all);
    // share `want` by cost with floors nmin and caps nbk (water filling, then
    // largest remainders)
    std::vector<double> share(ns, 0.0);
    std::vector<char> fixed(ns, 0);
    for (int iter = 0; iter < ns + 1; ++iter) {
        double free_cost = 0.0;
        long long free_ctas = want;
        for (int k = 0; k < ns; ++k) {
            if (fixed[k]) free_ctas -= (long long)share[k];
            else free_cost += cum[k][nbk[k]];
        }
        bool changed = false;
        for (int k = 0; k < ns; ++k) {
            if (fixed[k]) continue;
            share[k] = free_cost > 0 ? (double)free_ctas * cum[k][nbk[k]] / free_cost : 0.0;
            if (share[k] < nmin[k]) { share[k] = nmin[k]; fixed[k] = 1; changed = true; }
            else if (share[k] > (double)nbk[k]) { share[k] = (double)nbk[k]; fixed[k] = 1; changed = true; }
        }
        if (!changed) break;
    }
    std::vector<int> nc(ns);
    long long used = 0;
    std::vector<std::pair<double, int>> rem;
    for (int k = 0; k < ns; ++k) {
        nc[k] = std::max(nmin[k], (int)std::floor(share[k]));
        used += nc[k];
        rem.push_back({share[k] - std::floor(share[k]), k});
    }
    std::sort(rem.begin(), rem.end(), [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
        return a.first > b.first || (a.first == b.first && a.second < b.second);
    });
    for (size_t i = 0; i < rem.size() && used < want; ++i) {
        const int k = rem[i].second;
        if (nc[k] < nbk[k]) { ++nc[k]; ++used; }
    }
    plan.items.clear();
    plan.off.assign(1, 0);
    plan.cta0.assign(ns, 0);
    plan.ncta.assign(ns, 0);
    std::vector<long long> ends;
    for (int k = 0; k < ns; ++k) {
        plan.cta0[k] = (int)plan.off.size() - 1;
        if (nbk[k] == 0) continue;  // nothing to do for this shot
        if (tp.bands && !live &&
            cut_bands(cum[k], k, geo[k].xoff, strips_of(geo[k], tile_x), nzb[k], tile_x, nc[k], plan)) {
            plan.ncta[k] = (int)plan.off.size() - 1 - plan.cta0[k];
            continue;
        }
        int n = nc[k];
        while (!cut_shot(cum[k], nbk[k], run_of[k], run_begin[k], n, ends)) {
            if (n >= nbk[k]) return FD23_ERR_ARG;
            ++n;
        }
        plan.ncta[k] = n;
        long long b0 = 0;
        for (long long b1 : ends) {
            while (b0 < b1) {
                // one item per run inside the range
                const long long r = run_of[k][b0];
                const long long rend = r + 1 < (long long)run_begin[k].size() ? run_begin[k][r + 1] : nbk[k];
                const long long e = std::min(b1, rend);
                const long long first = blk[k][b0], last = blk[k][e - 1];
                const int strip = (int)(first / nzb[k]);
                plan.items.push_back(
                    WorkItem{k, geo[k].xoff + strip * tile_x, (int)(first % nzb[k]) * 4, (int)(last % nzb[k] + 1) * 4});
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
