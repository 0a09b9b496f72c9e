// Batched multi-shot sweep and the work-plan autotuner.
//
// A batch advances many solvers (shots of any grid size, one wave type and
// one precision, on one GPU) in lockstep: every time step is ONE launch of the
// fused sweep over all shots, driven by a work plan whose CTAs each serve one
// shot (fd23_plan.cpp) and a device table of shot descriptors.  The launches
// of a run are captured once into a CUDA graph and replayed; a run with the
// same step range, record pattern and plan replays the cached graph.
//
// The reference runs one shot per process (PD/main.cpp:43-183); this has no
// counterpart there.
//
// The autotuner times candidate work plans (block cost weights, CTAs per SM,
// oversubscription) on the live shots for a few steps each, restoring the
// wavefields, memory variables and step counters after every trial, and keeps
// the fastest plan.
#include <algorithm>
#include <new>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fd23_solver.h"

using namespace fd23;

struct fd23_batch {
    std::vector<fd23_solver *> s;
    int wave = 0, prec = 0, device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    TuneParams tune;
    WorkPlan plan;
    WorkItem *d_items = nullptr;
    int *d_off = nullptr;
    void *d_shots = nullptr;
    int *err_flag = nullptr;
    int plan_ver = 0;
    // cached graph of the last run: key = it0, nsteps, itrecord, par0, nrec0, plan version
    cudaGraphExec_t gexec = nullptr;
    long long gkey[7] = {-1, -1, -1, -1, -1, -1, -1};
    int use_graph = 1;
};

namespace {

int batch_plan(fd23_batch *b, const TuneParams &tp)
{
    std::vector<ShotGeom> geo;
    for (auto *s : b->s) geo.push_back(ShotGeom{s->d.nx, s->d.nz, s->d.npml, s->d.topabsorb});
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
    TuneParams t = tp;
    t.per_sm = std::min(t.per_sm, fused_per_sm(b->device, b->wave, b->prec, true));
    WorkPlan plan;
    int rc = plan_work(geo, fused_geom(b->wave, b->prec).tile_x, sms, t, plan);
    if (rc) return rc;
    if ((rc = upload_plan(plan, &b->d_items, &b->d_off))) return rc;
    b->plan = plan;
    b->tune = tp;
    ++b->plan_ver;
    return FD23_OK;
}

template <class S, class C>
int upload_shots(fd23_batch *b)
{
    std::vector<Shot<S, C>> t(b->s.size());
    for (size_t k = 0; k < b->s.size(); ++k) {
        t[k] = make_shot<S, C>(b->s[k]);
        t[k].cta0 = b->plan.cta0[k];
        t[k].ncta = b->plan.ncta[k];
    }
    if (!b->d_shots) {
        const int rc = dev_alloc(&b->d_shots, t.size() * sizeof(Shot<S, C>));
        if (rc) return rc;
    }
    CK(cudaMemcpyAsync(b->d_shots, t.data(), t.size() * sizeof(Shot<S, C>), cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return FD23_OK;
}

// the batch stream waits for every solver's queued work
int join_in(fd23_batch *b)
{
    for (auto *s : b->s) {
        CK(cudaEventRecord(b->ev, s->stream));
        CK(cudaStreamWaitEvent(b->stream, b->ev, 0));
    }
    return FD23_OK;
}
// every solver stream waits for the batch's queued work
int join_out(fd23_batch *b)
{
    CK(cudaEventRecord(b->ev, b->stream));
    for (auto *s : b->s) CK(cudaStreamWaitEvent(s->stream, b->ev, 0));
    return FD23_OK;
}

// launches of nsteps lockstep steps from (it, par, pending); returns the new
// pending record row through *pending
template <class S, class C>
int launch_steps(fd23_batch *b, int it0, int nsteps, int itrecord, bool any_rec, int par0, int nrec0,
                 bool punch, int *pending)
{
    const Shot<S, C> *shots = (const Shot<S, C> *)b->d_shots;
    int par = par0, pend = -1, nrec = nrec0;
    for (int k = 0; k < nsteps; ++k) {
        const int it = it0 + k;
        const int rc = launch_step_fused_batch<S, C>(shots, b->wave, b->d_items, b->d_off, b->plan.nblocks, par,
                                                     it, pend, b->err_flag, punch, b->s[0]->table_on, b->stream);
        if (rc) return rc;
        pend = (any_rec && it % itrecord == 0) ? nrec++ : -1;
        par = 1 - par;
    }
    *pending = pend;
    return FD23_OK;
}

template <class S, class C>
int batch_run_impl(fd23_batch *b, int nsteps, int itrecord)
{
    fd23_solver *s0 = b->s[0];
    for (auto *s : b->s) {
        if (!s->have_material) return FD23_ERR_ORDER;
        if (s->box_on || !s->fused) return FD23_ERR_UNSUPPORTED;
        if (s->it != s0->it || s->par != s0->par || s->nrec_steps != s0->nrec_steps || s->pending_rec >= 0)
            return FD23_ERR_ORDER;  // shots must be in lockstep
        int rc = ensure_sigma(s);
        if (rc) return rc;
    }
    int nrec_new = 0;
    for (int k = 0; k < nsteps; ++k)
        if ((s0->it + k) % itrecord == 0) ++nrec_new;
    bool any_rec = false, punch = false;
    for (auto *s : b->s) {
        for (int c = 0; c < 5; ++c) any_rec = any_rec || s->nrec[c] > 0;
        punch = punch || s->d_punch != nullptr;
        if (s->table_on != s0->table_on) return FD23_ERR_UNSUPPORTED;  // tables in all shots or none
    }
    if (any_rec)
        for (auto *s : b->s) {
            const int rc = ensure_record_capacity(s, s->nrec_steps + nrec_new);
            if (rc) return rc;
        }
    int rc = join_in(b);
    if (rc) return rc;
    if ((rc = upload_shots<S, C>(b))) return rc;
    const int it0 = s0->it, par0 = s0->par, nrec0 = s0->nrec_steps;
    int pending = -1;
    const long long key[7] = {it0, nsteps, itrecord * (any_rec ? 1 : -1), par0, nrec0, b->plan_ver,
                              (long long)punch + 2 * (long long)s0->table_on};
    bool done = false;
    if (b->use_graph && nsteps >= 2) {
        if (b->gexec && std::equal(key, key + 7, b->gkey)) {
            // replay; the pending record row follows from the key
            int nr = nrec0;
            for (int k = 0; k < nsteps; ++k) pending = (any_rec && (it0 + k) % itrecord == 0) ? nr++ : -1;
            done = cudaGraphLaunch(b->gexec, b->stream) == cudaSuccess;
            if (!done) cudaGetLastError();
        } else {
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                const int lr = launch_steps<S, C>(b, it0, nsteps, itrecord, any_rec, par0, nrec0, punch, &pending);
                const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
                cudaGraphExec_t ex = nullptr;
                if (lr == FD23_OK && ec == cudaSuccess && g &&
                    cudaGraphInstantiate(&ex, g, 0) == cudaSuccess && cudaGraphLaunch(ex, b->stream) == cudaSuccess) {
                    if (b->gexec) cudaGraphExecDestroy(b->gexec);
                    b->gexec = ex;
                    std::copy(key, key + 7, b->gkey);
                    done = true;
                } else if (ex) {
                    cudaGraphExecDestroy(ex);
                }
                if (g) cudaGraphDestroy(g);
            }
            if (!done) cudaGetLastError();  // capture unavailable: launch directly
        }
    }
    if (!done && (rc = launch_steps<S, C>(b, it0, nsteps, itrecord, any_rec, par0, nrec0, punch, &pending)))
        return rc;
    const int par1 = (nsteps & 1) ? 1 - par0 : par0;
    int nrec1 = nrec0;
    for (int k = 0; k < nsteps; ++k)
        if (any_rec && (it0 + k) % itrecord == 0) ++nrec1;
    for (auto *s : b->s) {
        s->it = it0 + nsteps;
        s->par = par1;
        s->nrec_steps = nrec1;
        s->pending_rec = -1;
        if (pending >= 0 && (rc = launch_record<S, C>(make_shot<S, C>(s), par1, pending, b->stream))) return rc;
    }
    return join_out(b);
}

int batch_run(fd23_batch *b, int nsteps, int itrecord)
{
    switch (b->prec) {
        case FD23_F64: return batch_run_impl<double, double>(b, nsteps, itrecord);
        case FD23_BF16: return batch_run_impl<__nv_bfloat16, float>(b, nsteps, itrecord);
        case FD23_F16: return batch_run_impl<__half, float>(b, nsteps, itrecord);
        default: return batch_run_impl<float, float>(b, nsteps, itrecord);
    }
}

// ---- autotuner ----

// state of the solvers (read set of wavefields, memory variables, box
// residual, step counters) saved before trials and put back after each
struct Snapshot {
    std::vector<void *> copy, live;
    std::vector<size_t> bytes;
    std::vector<int> it, par, nrec, pend;
    ~Snapshot()
    {
        for (void *p : copy) cudaFree(p);
    }
};

int snapshot_take(const std::vector<fd23_solver *> &ss, cudaStream_t st, Snapshot &sn)
{
    for (auto *s : ss) {
        auto add = [&](void *p, size_t n) -> int {
            if (!p || !n) return FD23_OK;
            void *c = nullptr;
            const int rc = dev_alloc(&c, n);
            if (rc) return rc;
            sn.copy.push_back(c);
            sn.live.push_back(p);
            sn.bytes.push_back(n);
            CK(cudaMemcpyAsync(c, p, n, cudaMemcpyDeviceToDevice, st));
            return FD23_OK;
        };
        int rc = FD23_OK;
        for (int f = 0; f < s->nfld && !rc; ++f) rc = add(s->fld[s->par][f], s->L.elems() * s->es);
        for (int p = 0; p < s->npsi && !rc; ++p) rc = add(s->psi[s->par][p], s->psi_elems[p] * s->cs);
        if (s->box_on)
            for (int f = 0; f < 5 && !rc; ++f) rc = add(s->box_r[f], (size_t)s->box_bx * s->box_bz * s->cs);
        if (rc) return rc;
        sn.it.push_back(s->it);
        sn.par.push_back(s->par);
        sn.nrec.push_back(s->nrec_steps);
        sn.pend.push_back(s->pending_rec);
    }
    CK(cudaStreamSynchronize(st));
    return FD23_OK;
}

int snapshot_restore(const std::vector<fd23_solver *> &ss, cudaStream_t st, const Snapshot &sn)
{
    for (size_t k = 0; k < ss.size(); ++k) {
        ss[k]->it = sn.it[k];
        ss[k]->par = sn.par[k];
        ss[k]->nrec_steps = sn.nrec[k];
        ss[k]->pending_rec = sn.pend[k];
    }
    for (size_t i = 0; i < sn.copy.size(); ++i)
        CK(cudaMemcpyAsync(sn.live[i], sn.copy[i], sn.bytes[i], cudaMemcpyDeviceToDevice, st));
    // the trial steps wrote the other set: with tile step windows the sweep
    // relies on both sets agreeing on the tiles it leaves alone
    for (auto *s : ss)
        if (s->d_punch) {
            const int rc = mirror_sets(s, st);
            if (rc) return rc;
        }
    CK(cudaStreamSynchronize(st));
    return FD23_OK;
}

// block cost weights (x-CPML 2..7, z-CPML and edge rows 2..5) x waves of
// CTAs 1..3 (the plan rounds the CTA count up to whole waves of the resident
// slots) x the two ways of cutting (strip after strip, or banded): the step
// time is a bumpy function of the cut, so the grid is fine (on the
// 4000 x 2000 P-SV grid weights 5 / 4 beat 6 / 4 by 6 %)
std::vector<TuneParams> candidates()
{
    std::vector<TuneParams> c;
    for (int bands : {0, 1})
        for (double ov : {1.0, 2.0, 3.0})
            for (double wx : {2.0, 3.0, 4.0, 5.0, 6.0, 7.0})
                for (double wz : {2.0, 3.0, 4.0, 5.0}) {
                    TuneParams t;
                    t.wx = wx;
                    t.wz = wz;
                    t.oversub = ov;
                    t.bands = bands;
                    c.push_back(t);
                }
    return c;
}

// Times every candidate for trial_steps steps, then the five fastest again
// for three times as long (short trials are noisy), then the half-step
// neighbours of the best weights; keeps the best of the long trials
// installed.  `apply` installs a plan, `steps` runs k steps without
// recording on `st`.  The table gets every trial, the second round last.
template <class Apply, class Steps>
int autotune_core(const std::vector<fd23_solver *> &ss, cudaStream_t st, int trial_steps, Apply apply,
                  Steps steps, fd23_tune_entry *table, int cap, bool try_fast)
{
    Snapshot sn;
    int rc = snapshot_take(ss, st, sn);
    if (rc) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    std::vector<TuneParams> cand = candidates();
    int best = -1, n = 0;
    std::vector<double> first(cand.size(), 1e300);
    auto trial = [&](size_t i, int k, double *per) -> int {
        int r = apply(cand[i]);
        if (!r) r = steps(2);  // warm-up
        if (r) return r;
        CK(cudaEventRecord(e0, st));
        if ((r = steps(k))) return r;
        CK(cudaEventRecord(e1, st));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        *per = ms / k;
        if (table && n < cap)
            table[n] = fd23_tune_entry{cand[i].wx,    cand[i].wz, cand[i].per_sm, cand[i].bands,
                                       cand[i].oversub, *per,     cand[i].fast};
        ++n;
        return snapshot_restore(ss, st, sn);
    };
    for (size_t i = 0; i < cand.size() && !rc; ++i) rc = trial(i, trial_steps, &first[i]);
    if (!rc) {
        std::vector<size_t> order(cand.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return first[a] < first[b]; });
        double best_ms = 0.0;
        for (size_t k = 0; k < std::min<size_t>(5, order.size()) && !rc; ++k) {
            double per = 0.0;
            rc = trial(order[k], 3 * trial_steps, &per);
            if (!rc && (best < 0 || per < best_ms)) {
                best = (int)order[k];
                best_ms = per;
            }
        }
        // third round: the half-step neighbours of the best weights
        const TuneParams b0 = cand[best];
        for (double dx : {-0.5, 0.0, 0.5})
            for (double dz : {-0.5, 0.0, 0.5}) {
                if ((dx == 0.0 && dz == 0.0) || b0.wx + dx < 1.0 || b0.wz + dz < 1.0 || rc) continue;
                TuneParams t = b0;
                t.wx += dx;
                t.wz += dz;
                cand.push_back(t);
                double per = 0.0;
                rc = trial(cand.size() - 1, 3 * trial_steps, &per);
                if (!rc && per < best_ms) {
                    best = (int)cand.size() - 1;
                    best_ms = per;
                }
            }
        // last: the best plan on the sweep instantiation with fast iterations
        if (try_fast && !rc) {
            TuneParams t = cand[best];
            t.fast = 1;
            cand.push_back(t);
            double per = 0.0;
            rc = trial(cand.size() - 1, 3 * trial_steps, &per);
            if (!rc && per < best_ms) {
                best = (int)cand.size() - 1;
                best_ms = per;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) {
        snapshot_restore(ss, st, sn);
        return rc;
    }
    if ((rc = apply(cand[best]))) return rc;
    return n;
}

}  // namespace

extern "C" {

int fd23_batch_create(fd23_solver *const *solvers, int n, fd23_batch **out)
{
    if (!solvers || n <= 0 || !out) return FD23_ERR_ARG;
    *out = nullptr;
    fd23_solver *s0 = solvers[0];
    if (!s0) return FD23_ERR_ARG;
    for (int k = 0; k < n; ++k) {
        fd23_solver *s = solvers[k];
        if (!s || s->d.wave != s0->d.wave || s->d.prec != s0->d.prec || s->d.device != s0->d.device)
            return FD23_ERR_ARG;
        for (int j = 0; j < k; ++j)
            if (solvers[j] == s) return FD23_ERR_ARG;
        if (!s->fused) return FD23_ERR_UNSUPPORTED;
    }
    CK(cudaSetDevice(s0->d.device));
    fd23_batch *b = new (std::nothrow) fd23_batch();
    if (!b) return FD23_ERR_NOMEM;
    b->s.assign(solvers, solvers + n);
    b->wave = s0->d.wave;
    b->prec = s0->d.prec;
    b->device = s0->d.device;
    b->tune = s0->tune;
    int rc = FD23_OK;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        rc = FD23_ERR_CUDA;
    }
    if (!rc) rc = dev_alloc((void **)&b->err_flag, sizeof(int));
    if (!rc && cudaMemset(b->err_flag, 0, sizeof(int)) != cudaSuccess) rc = FD23_ERR_CUDA;
    if (!rc) rc = batch_plan(b, b->tune);
    if (rc) {
        fd23_batch_destroy(b);
        return rc;
    }
    *out = b;
    return FD23_OK;
}

void fd23_batch_destroy(fd23_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    cudaFree(b->d_items);
    cudaFree(b->d_off);
    cudaFree(b->d_shots);
    cudaFree(b->err_flag);
    if (b->ev) cudaEventDestroy(b->ev);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int fd23_batch_run(fd23_batch *b, int nsteps, int itrecord)
{
    if (!b || nsteps < 0 || itrecord <= 0) return FD23_ERR_ARG;
    CK(cudaSetDevice(b->device));
    if (nsteps == 0) return FD23_OK;
    return batch_run(b, nsteps, itrecord);
}

int fd23_batch_sync(fd23_batch *b)
{
    if (!b) return FD23_ERR_ARG;
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->stream));
    int flag = 0;
    CK(cudaMemcpy(&flag, b->err_flag, sizeof(int), cudaMemcpyDeviceToHost));
    return flag ? FD23_ERR_TIMEOUT : FD23_OK;
}

int fd23_batch_get_stream(fd23_batch *b, void **stream)
{
    if (!b || !stream) return FD23_ERR_ARG;
    *stream = (void *)b->stream;
    return FD23_OK;
}

int fd23_batch_set_graph(fd23_batch *b, int on)
{
    if (!b) return FD23_ERR_ARG;
    b->use_graph = on ? 1 : 0;
    return FD23_OK;
}

int fd23_batch_set_plan(fd23_batch *b, const fd23_tune_entry *tune)
{
    if (!b || !tune || !(tune->wx > 0) || !(tune->wz > 0) || tune->per_sm < 1 || !(tune->oversub >= 1.0 / 16) ||
        tune->oversub > 64.0 || (tune->bands != 0 && tune->bands != 1) || (tune->fast_iter != 0 && tune->fast_iter != 1))
        return FD23_ERR_ARG;
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->stream));  // the old work list may still be in use
    TuneParams t{tune->wx, tune->wz, tune->per_sm, tune->oversub, tune->bands};
    return batch_plan(b, t);
}

int fd23_batch_get_plan(fd23_batch *b, fd23_tune_entry *cur, int *nblocks)
{
    if (!b) return FD23_ERR_ARG;
    if (cur) *cur = fd23_tune_entry{b->tune.wx, b->tune.wz, b->tune.per_sm, b->tune.bands, b->tune.oversub, 0.0, 0};
    if (nblocks) *nblocks = b->plan.nblocks;
    return FD23_OK;
}

int fd23_batch_autotune(fd23_batch *b, int trial_steps, fd23_tune_entry *table, int cap)
{
    if (!b || trial_steps <= 0 || cap < 0 || (cap > 0 && !table)) return FD23_ERR_ARG;
    CK(cudaSetDevice(b->device));
    fd23_solver *s0 = b->s[0];
    for (auto *s : b->s) {
        if (!s->have_material) return FD23_ERR_ORDER;
        if (s->it != s0->it || s->par != s0->par || s->pending_rec >= 0) return FD23_ERR_ORDER;
        if (s->table_on != s0->table_on) return FD23_ERR_UNSUPPORTED;  // tables in all shots or none
        const int rc = ensure_sigma(s);
        if (rc) return rc;
    }
    int rc = join_in(b);
    if (rc) return rc;
    auto apply = [b](const TuneParams &tp) -> int {
        const int r = batch_plan(b, tp);
        if (r) return r;
        switch (b->prec) {
            case FD23_F64: return upload_shots<double, double>(b);
            case FD23_BF16: return upload_shots<__nv_bfloat16, float>(b);
            case FD23_F16: return upload_shots<__half, float>(b);
            default: return upload_shots<float, float>(b);
        }
    };
    bool punch = false;
    for (auto *s : b->s) punch = punch || s->d_punch != nullptr;
    auto steps = [b, punch](int k) -> int {
        fd23_solver *s = b->s[0];
        int pend = -1;
        int r;
        switch (b->prec) {
            case FD23_F64: r = launch_steps<double, double>(b, s->it, k, 1, false, s->par, 0, punch, &pend); break;
            case FD23_BF16: r = launch_steps<__nv_bfloat16, float>(b, s->it, k, 1, false, s->par, 0, punch, &pend); break;
            case FD23_F16: r = launch_steps<__half, float>(b, s->it, k, 1, false, s->par, 0, punch, &pend); break;
            default: r = launch_steps<float, float>(b, s->it, k, 1, false, s->par, 0, punch, &pend);
        }
        if (r) return r;
        for (auto *x : b->s) {
            x->it += k;
            x->par = (k & 1) ? 1 - x->par : x->par;
        }
        return FD23_OK;
    };
    rc = autotune_core(b->s, b->stream, trial_steps, apply, steps, table, cap, false);
    const int jr = join_out(b);
    return rc < 0 ? rc : (jr ? jr : rc);
}

int fd23_work_plan_live(int nshots, const int *nx, const int *nz, const int *npml, const int *topabsorb, int sms,
                        const fd23_tune_entry *tune, const unsigned char *live, int *items, int cap_items, int *off,
                        int cap_ctas)
{
    if (nshots <= 0 || !nx || !nz || !npml || !topabsorb || sms <= 0 || !tune || !items || !off) return FD23_ERR_ARG;
    std::vector<ShotGeom> geo;
    for (int k = 0; k < nshots; ++k) {
        if (nx[k] < 2 || nz[k] < 2 || npml[k] < 0) return FD23_ERR_ARG;
        geo.push_back(ShotGeom{nx[k], nz[k], npml[k], topabsorb[k]});
    }
    TuneParams tp;
    tp.wx = tune->wx;
    tp.wz = tune->wz;
    tp.per_sm = tune->per_sm;
    tp.oversub = tune->oversub;
    tp.bands = tune->bands;
    const int tx = fused_geom(FD23_PSV, FD23_F32).tile_x;
    std::vector<std::vector<unsigned char>> masks;
    if (live) {
        size_t at = 0;
        for (int k = 0; k < nshots; ++k) {
            const size_t nb = (size_t)((nx[k] + tx - 1) / tx) * ((nz[k] + 3) / 4);
            masks.emplace_back(live + at, live + at + nb);
            at += nb;
        }
    }
    WorkPlan plan;
    const int rc = plan_work(geo, tx, sms, tp, plan, live ? &masks : nullptr);
    if (rc) return rc;
    if ((int)plan.items.size() > cap_items || plan.nblocks + 1 > cap_ctas + 1) return FD23_ERR_ARG;
    for (size_t i = 0; i < plan.items.size(); ++i) {
        items[4 * i] = plan.items[i].shot;
        items[4 * i + 1] = plan.items[i].x0;
        items[4 * i + 2] = plan.items[i].z0;
        items[4 * i + 3] = plan.items[i].z1;
    }
    for (int c = 0; c <= plan.nblocks; ++c) off[c] = plan.off[c];
    return plan.nblocks;
}

int fd23_work_plan(int nshots, const int *nx, const int *nz, const int *npml, const int *topabsorb, int sms,
                   const fd23_tune_entry *tune, int *items, int cap_items, int *off, int cap_ctas)
{
    return fd23_work_plan_live(nshots, nx, nz, npml, topabsorb, sms, tune, nullptr, items, cap_items, off, cap_ctas);
}

int fd23_set_plan(fd23_solver *s, const fd23_tune_entry *tune)
{
    if (!s || !tune || !(tune->wx > 0) || !(tune->wz > 0) || tune->per_sm < 1 || !(tune->oversub >= 1.0 / 16) ||
        tune->oversub > 64.0 || (tune->bands != 0 && tune->bands != 1) || (tune->fast_iter != 0 && tune->fast_iter != 1))
        return FD23_ERR_ARG;
    if (!s->fused) return FD23_ERR_UNSUPPORTED;
    CK(cudaSetDevice(s->d.device));
    CK(cudaStreamSynchronize(s->stream));  // the old work list may still be in use
    TuneParams t{tune->wx, tune->wz, tune->per_sm, tune->oversub, tune->bands};
    t.shift = s->tune.shift;
    t.fast = tune->fast_iter;
    s->tune = t;
    int rc = build_worklist(s);
    // the two-step sweep's plan takes the same weights and cut (its own CTAs per SM)
    if (!rc && s->fused2) rc = build_worklist2(s);
    return rc;
}

int fd23_get_plan(fd23_solver *s, fd23_tune_entry *cur, int *nblocks)
{
    if (!s) return FD23_ERR_ARG;
    if (cur)
        *cur = fd23_tune_entry{s->tune.wx, s->tune.wz, s->tune.per_sm, s->tune.bands, s->tune.oversub, 0.0,
                               s->tune.fast};
    if (nblocks) *nblocks = s->nblocks;
    return FD23_OK;
}

int fd23_autotune(fd23_solver *s, int trial_steps, fd23_tune_entry *table, int cap)
{
    if (!s || trial_steps <= 0 || cap < 0 || (cap > 0 && !table)) return FD23_ERR_ARG;
    if (!s->fused) return FD23_ERR_UNSUPPORTED;
    if (!s->have_material) return FD23_ERR_ORDER;
    CK(cudaSetDevice(s->d.device));
    int rc = ensure_sigma(s);
    if (rc) return rc;
    if (s->box_on && (s->it < s->box_inc_it0 || s->it + trial_steps + 2 > s->box_inc_it0 + s->box_inc_n))
        return FD23_ERR_ORDER;
    if ((rc = dispatch_flush(s))) return rc;
    std::vector<fd23_solver *> ss{s};
    auto apply = [s](const TuneParams &tp) -> int {
        s->tune = tp;
        return build_worklist(s);
    };
    auto steps = [s](int k) -> int {
        for (int i = 0; i < k; ++i) {
            const int r = dispatch_step(s, 0);
            if (r) return r;
        }
        return FD23_OK;
    };
    // the fast-iteration instantiation exists for the plain FP32 sweep only
    // (window, table and box runs launch other sweeps, which ignore it)
    const bool try_fast = s->d.prec == FD23_F32 && !s->d_punch && !s->d_midx && !s->box_on;
    return autotune_core(ss, s->stream, trial_steps, apply, steps, table, cap, try_fast);
}

}  // extern "C"
