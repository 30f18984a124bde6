/*
 * Groups: many structures of uneven size (each an FP32 plan with its own batch
 * of excitations) advanced together, one CUDA graph launch per 32 steps.
 *
 * The reference runs one structure per process (FDTDcalc/FDTDsplitfieldMetal.c
 * main); an S-matrix sweep over a family of structures is a loop of such
 * runs.  Here the member plans keep their own device state, schedule, sources
 * and DFT; the group replaces their per-step launches, in one of two modes:
 *   0: one grouped launch per sweep over the cells of every member
 *      (k_group32v: a block finds its member by prefix sums in a
 *      constant-memory table; one such group per device at a time, so
 *      group_run holds a lock and completes before returning in this mode);
 *   1: each member's own vectorised-sweep launches, back to back on the
 *      group's stream;
 *   2: each member's own tuned launch form on its own stream (forked from the
 *      group's stream and joined back);
 *   3: one persistent launch of the whole-row fused step per step over every
 *      member (k_row32g): the resident CTAs are shared out among the members
 *      in groups of one CTA per excitation, each member's groups marching its
 *      own persistent schedule;
 * always captured as one CUDA graph per 32 steps, with each member's DFT
 * ring flushed in it.  Member results are bit-identical to stepping each
 * plan alone.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "trace.cuh"
#include "plan_internal.cuh"

using namespace smat;
using namespace smat::plan;

struct smat_fdtd_group {
    std::vector<smat_fdtd_plan *> m;
    std::vector<int> cur; /* members' field sets when the graph was captured */
    Group32 *h_gr = nullptr; /* pinned copy of the member table (mode 0) */
    cudaStream_t stream = nullptr;
    int mode = 0; /* 0: one grouped launch per sweep; 1: each member's own sweep launches;
                     2: each member's own launch form, on its own stream;
                     3: one persistent fused launch over every member */
    int by = 1;   /* modes 0, 1: rows per block; mode 3: 1 = CTAs of 384 threads, 2 = of 192 */
    /* mode 3: members' rows per tile and CTA groups, the launch's shape */
    std::vector<int> ty3, groups3;
    int grid3 = 0, threads3 = 384;
    size_t smem3 = 0;
    bool rec3 = false;
    cudaEvent_t fork = nullptr;      /* mode 2: members' streams wait for the group's stream ... */
    std::vector<cudaEvent_t> join;   /* ... and the group's stream for each member's */
    cudaGraphExec_t graph = nullptr;
    bool graph_failed = false;
};

namespace {

std::mutex g_table_mu; /* the constant-memory member table of mode 0 */

Group32 make_group(const smat_fdtd_group *g)
{
    Group32 gr;
    memset(&gr, 0, sizeof gr);
    gr.n = (int)g->m.size();
    gr.by = g->by;
    int blk = 0, gh = 0, ge = 0;
    for (int i = 0; i < gr.n; i++) {
        smat_fdtd_plan *p = g->m[i];
        gr.blk[i] = blk;
        gr.gen_h[i] = gh;
        gr.gen_e[i] = ge;
        gr.p[i] = make_p32(p, false);
        gr.hgen[i] = p->d_hgen;
        gr.egen[i] = p->d_egen;
        gr.nhgen[i] = p->nhgen;
        gr.negen[i] = p->negen;
        const int nxb = (p->L[0] / 4 + 31) / 32;
        blk += nxb * ((p->L[1] + g->by - 1) / g->by) * p->batch * p->L[2];
        gh += p->nhgen * p->batch;
        ge += p->negen * p->batch;
    }
    gr.blk[gr.n] = blk;
    gr.gen_h[gr.n] = gh;
    gr.gen_e[gr.n] = ge;
    return gr;
}

/* Mode 3's shape for CTAs of `threads` threads (384: one per SM, 192: two).
 * Each member's tile is the most whole rows (up to 16) whose quads fit the
 * CTA and whose staging fits the CTA's share of shared memory.  The resident
 * CTAs are shared out in groups of one CTA per excitation: every member gets
 * one group, then each further group goes to the member with the most cells
 * per CTA while CTAs are left. */
int setup_persistent(smat_fdtd_group *g, int threads)
{
    const size_t room = threads == 384 ? 232448 : 232448 / 2 - 1024;
    const int n = (int)g->m.size();
    std::vector<int> ty(n), groups(n, 1);
    size_t smem = 0;
    bool rec = false;
    int used = 0;
    for (int i = 0; i < n; i++) {
        const smat_fdtd_plan *p = g->m[i];
        const int nq = p->L[0] / 4;
        int t = 0;
        for (int c = 16; c >= 1 && !t; c--)
            if (nq * (c + 1) <= threads && row32_smem(p->L[0], c, p->L[2]) <= room) t = c;
        if (!t)
            return smat_fail(SMAT_EINVAL, "group_set_tuning: member %d's rows of %d cells do not fit mode 3's CTA",
                             i, p->L[0]);
        ty[i] = t;
        smem = std::max(smem, row32_smem(p->L[0], t, p->L[2]));
        rec |= p->nhgen + p->negen > 0;
        used += p->batch;
    }
    const int occ = row32_group_max_ctas_per_sm(threads, smem, rec);
    if (occ < 1) return smat_fail(SMAT_EINVAL, "group_set_tuning: mode 3 does not fit an SM");
    const int total = sm_count() * occ;
    if (used > total)
        return smat_fail(SMAT_EINVAL, "group_set_tuning: mode 3 needs a CTA per excitation (%d) within the %d "
                                      "resident CTAs", used, total);
    std::vector<double> cells(n);
    for (int i = 0; i < n; i++) {
        const smat_fdtd_plan *p = g->m[i];
        cells[i] = (double)p->L[0] * p->L[1] * p->L[2];
    }
    for (;;) {
        int best = -1;
        double load = 0;
        for (int i = 0; i < n; i++) {
            const double l = cells[i] / groups[i]; /* per CTA of the member */
            if (used + g->m[i]->batch <= total && l > load) {
                load = l;
                best = i;
            }
        }
        if (best < 0) break;
        groups[best]++;
        used += g->m[best]->batch;
    }
    g->ty3 = ty;
    g->groups3 = groups;
    g->smem3 = smem;
    g->rec3 = rec;
    g->grid3 = used;
    g->threads3 = threads;
    return SMAT_OK;
}

/* the mode and block_y of set_tuning (mode 3 builds its piece list) */
int configure(smat_fdtd_group *g, int mode, int by)
{
    if (mode == 3) {
        if (by != 1 && by != 2) return smat_fail(SMAT_EINVAL, "group_set_tuning: mode 3 takes block_y 1 or 2");
        int rc = setup_persistent(g, by == 1 ? 384 : 192);
        if (rc) return rc;
    }
    g->mode = mode;
    g->by = by;
    return SMAT_OK;
}

/* steps rel0 .. rel0+n-1 of every member (relative to each member's d_base) */
void enqueue_group(smat_fdtd_group *g, int rel0, int n)
{
    if (g->mode == 3) {
        /* one persistent launch a step: each member's groups of CTAs */
        RowGroup32 G;
        memset(&G, 0, sizeof G);
        G.n = (int)g->m.size();
        int first = 0;
        for (int j = 0; j < G.n; j++) {
            G.first[j] = first;
            first += g->groups3[j] * g->m[j]->batch;
        }
        G.first[G.n] = first;
        for (int i = 0; i < n; i++) {
            for (int j = 0; j < G.n; j++) {
                const smat_fdtd_plan *p = g->m[j];
                Row32 &r = G.r[j];
                r = make_row(p, false);
                r.ty = g->ty3[j];
                r.zc = 0;
                r.nyt = (p->L[1] + g->ty3[j] - 1) / g->ty3[j];
                r.nzc = 1;
                r.ngroups = g->groups3[j];
                r.nitems = g->groups3[j] * p->batch;
                r.worder = 0;
            }
            launch_row32_group(G, rel0 + i, g->threads3, g->grid3, g->smem3, g->rec3, g->stream);
            /* members with metal cells: their second launch, before the sets swap */
            for (int j = 0; j < G.n; j++) {
                const smat_fdtd_plan *p = g->m[j];
                launch_row_metal(G.r[j], rel0 + i, p->d_hmetal, p->nhmetal, p->d_emetal, p->nemetal, g->stream);
            }
            for (smat_fdtd_plan *p : g->m) p->cur ^= 1;
        }
    } else if (g->mode == 0) {
        *g->h_gr = make_group(g); /* same bytes on every call while the members stand still */
        load_group32(g->h_gr, g->stream);
        for (int i = 0; i < n; i++) launch_group32v(*g->h_gr, rel0 + i, g->stream);
    } else if (g->mode == 2) {
        /* each member's own (autotuned) launch form and DFT flush on its own
         * stream, forked from the group's stream and joined back: the members
         * run side by side (one graph launch per chunk of steps) */
        cudaEventRecord(g->fork, g->stream);
        for (size_t j = 0; j < g->m.size(); j++) {
            smat_fdtd_plan *p = g->m[j];
            const cudaStream_t st = p->stream;
            if (st != g->stream) cudaStreamWaitEvent(st, g->fork, 0);
            for (int i = 0; i < n; i++) enqueue_update(p, rel0 + i, st);
            launch_flush32(make_p32(p, false), rel0 + n, n, st);
            if (st != g->stream) {
                cudaEventRecord(g->join[j], st);
                cudaStreamWaitEvent(g->stream, g->join[j], 0);
            }
        }
        return;
    } else {
        /* each member's own vectorised sweeps (rows g->by, whole grid), in
         * order on the group's stream: one graph launch per chunk of steps */
        for (int i = 0; i < n; i++)
            for (smat_fdtd_plan *p : g->m) {
                const int by = p->by32, szc = p->szc, fu = p->fused;
                p->by32 = g->by;
                p->szc = 0;
                p->fused = 2;
                sweep_step(p, make_p32(p, false), rel0 + i, g->stream);
                p->by32 = by;
                p->szc = szc;
                p->fused = fu;
            }
    }
    for (smat_fdtd_plan *p : g->m) launch_flush32(make_p32(p, false), rel0 + n, n, g->stream);
}

void drop_group_graph(smat_fdtd_group *g)
{
    if (g->graph) cudaGraphExecDestroy(g->graph);
    g->graph = nullptr;
    g->graph_failed = false;
}

void build_group_graph(smat_fdtd_group *g)
{
    if (g->graph || g->graph_failed) return;
    cudaGraph_t gg = nullptr;
    if (cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        g->graph_failed = true;
        return;
    }
    enqueue_group(g, 0, GRAPH_STEPS);
    for (smat_fdtd_plan *p : g->m) launch_bump(p->d_base, GRAPH_STEPS, g->stream);
    g->cur.clear();
    for (smat_fdtd_plan *p : g->m) g->cur.push_back(p->cur);
    if (cudaStreamEndCapture(g->stream, &gg) != cudaSuccess || !gg) {
        cudaGetLastError();
        g->graph_failed = true;
        return;
    }
    if (cudaGraphInstantiate(&g->graph, gg, 0) != cudaSuccess) {
        cudaGetLastError();
        g->graph = nullptr;
        g->graph_failed = true;
    }
    cudaGraphDestroy(gg);
}

int sync_members(smat_fdtd_group *g)
{
    for (smat_fdtd_plan *p : g->m) CK(cudaStreamSynchronize(p->stream));
    return SMAT_OK;
}

} // namespace

extern "C" int smat_fdtd_group_create(smat_fdtd_plan *const *plans, int nplans, smat_fdtd_group **out)
{
    smat_clear_error();
    if (!plans || !out || nplans < 1) return smat_fail(SMAT_EINVAL, "group_create: bad arguments");
    if (nplans > MAX_GROUP) return smat_fail(SMAT_EINVAL, "group_create: at most %d plans per group", MAX_GROUP);
    *out = nullptr;
    for (int i = 0; i < nplans; i++) {
        const smat_fdtd_plan *p = plans[i];
        if (!p) return smat_fail(SMAT_EINVAL, "group_create: plan %d is null", i);
        if (p->precision != SMAT_FP32 || p->L[0] % 4 != 0)
            return smat_fail(SMAT_EINVAL, "group_create: plan %d is not an FP32 plan with L0 %% 4 == 0", i);
        for (int j = 0; j < i; j++)
            if (plans[j] == p) return smat_fail(SMAT_EINVAL, "group_create: plan %d appears twice", i);
    }
    smat_fdtd_group *g = new (std::nothrow) smat_fdtd_group();
    if (!g) return smat_fail(SMAT_ENOMEM, "group_create: out of host memory");
    if (cudaMallocHost((void **)&g->h_gr, sizeof(Group32)) != cudaSuccess) {
        cudaGetLastError();
        delete g;
        return smat_fail(SMAT_ENOMEM, "group_create: pinned host memory");
    }
    g->m.assign(plans, plans + nplans);
    g->stream = plans[0]->stream;
    g->join.assign(nplans, nullptr);
    bool ev_ok = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < nplans && ev_ok; i++)
        ev_ok = cudaEventCreateWithFlags(&g->join[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ev_ok) {
        cudaGetLastError();
        smat_fdtd_group_destroy(g);
        return smat_fail(SMAT_ECUDA, "group_create: events");
    }
    *out = g;
    return SMAT_OK;
}

extern "C" int smat_fdtd_group_destroy(smat_fdtd_group *g)
{
    if (!g) return SMAT_OK;
    if (g->stream) cudaStreamSynchronize(g->stream);
    drop_group_graph(g);
    if (g->h_gr) cudaFreeHost(g->h_gr);
    if (g->fork) cudaEventDestroy(g->fork);
    for (cudaEvent_t e : g->join)
        if (e) cudaEventDestroy(e);
    delete g;
    return SMAT_OK;
}

extern "C" int smat_fdtd_group_set_tuning(smat_fdtd_group *g, int mode, int block_y)
{
    smat_clear_error();
    if (!g || mode < 0 || mode > 3 || block_y < 1 || block_y > 4)
        return smat_fail(SMAT_EINVAL, "group_set_tuning: mode 0 (one launch per sweep), 1 (members' own sweep "
                                      "launches), 2 (members' own tuned launch forms) or 3 (one persistent fused "
                                      "launch), block_y in 1..4");
    if (g->stream) CK(cudaStreamSynchronize(g->stream));
    int rc = configure(g, mode, block_y);
    drop_group_graph(g);
    return rc;
}

extern "C" int smat_fdtd_group_run(smat_fdtd_group *g, int k_begin, int k_end)
{
    smat::TraceRange trace_("smat_fdtd_group_run");
    smat_clear_error();
    if (!g || k_begin < 0 || k_end < k_begin) return smat_fail(SMAT_EINVAL, "group_run: bad step range");
    for (size_t i = 0; i < g->m.size(); i++) {
        const smat_fdtd_plan *p = g->m[i];
        if (!p->d_sched) return smat_fail(SMAT_ESTATE, "group_run: member %zu has no schedule", i);
        if (k_end > p->nsched)
            return smat_fail(SMAT_EINVAL, "group_run: k_end %d beyond member %zu's %d-step schedule", k_end, i,
                             p->nsched);
    }
    /* mode 0 uses the device's one constant-memory member table: one such
     * group runs at a time (the run completes before the lock is released) */
    std::unique_lock<std::mutex> lock(g_table_mu, std::defer_lock);
    if (g->mode == 0) lock.lock();
    int rc = sync_members(g); /* members' own streams may still hold work */
    if (rc) return rc;
    /* a member stepped on its own with a fused kernel may have swapped field sets */
    for (size_t i = 0; i < g->cur.size() && i < g->m.size(); i++)
        if (g->cur[i] != g->m[i]->cur) {
            drop_group_graph(g);
            break;
        }
    for (smat_fdtd_plan *p : g->m) launch_set(p->d_base, k_begin, g->stream);
    int n = k_end - k_begin;
    if (n >= GRAPH_STEPS) build_group_graph(g);
    while (n >= GRAPH_STEPS) {
        if (g->graph) {
            CK(cudaGraphLaunch(g->graph, g->stream));
        } else {
            enqueue_group(g, 0, GRAPH_STEPS);
            for (smat_fdtd_plan *p : g->m) launch_bump(p->d_base, GRAPH_STEPS, g->stream);
        }
        n -= GRAPH_STEPS;
    }
    if (n > 0) {
        enqueue_group(g, 0, n);
        for (smat_fdtd_plan *p : g->m) launch_bump(p->d_base, n, g->stream);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "group_run: launch");
    if (g->mode == 0) CK(cudaStreamSynchronize(g->stream));
    return SMAT_OK;
}

extern "C" int smat_fdtd_group_sync(smat_fdtd_group *g)
{
    if (!g) return smat_fail(SMAT_EINVAL, "null group");
    CK(cudaStreamSynchronize(g->stream));
    for (smat_fdtd_plan *p : g->m) {
        int rc = smat_fdtd_sync(p);
        if (rc) return rc;
    }
    return SMAT_OK;
}

/* Times each mode and block_y over nsteps steps and keeps the fastest.  Like the plan
 * autotuner it needs every member at the zero state and runs with sources and
 * DFT sampling off, so the members are left as they were. */
extern "C" int smat_fdtd_group_autotune(smat_fdtd_group *g, int nsteps, int best[2], double *best_ms)
{
    smat_clear_error();
    if (!g || nsteps < 1) return smat_fail(SMAT_EINVAL, "group_autotune: bad arguments");
    for (smat_fdtd_plan *p : g->m) {
        int finite = 0;
        double mx = 0;
        int rc = smat_fdtd_check_finite(p, &finite, &mx);
        if (rc) return rc;
        if (mx != 0.0) return smat_fail(SMAT_ESTATE, "group_autotune: needs every member at the zero state");
    }
    /* form 2 steps each member in its own fastest launch form: tune them
     * (each on its own stream, sources and DFT off, back at the zero state) */
    for (smat_fdtd_plan *p : g->m) {
        int rc = smat_fdtd_autotune(p, nsteps, nullptr, nullptr);
        if (rc) return rc;
    }
    std::vector<int> nq(g->m.size());
    for (size_t i = 0; i < g->m.size(); i++) {
        smat_fdtd_plan *p = g->m[i];
        nq[i] = p->nq;
        p->nq = 0;
        CK(cudaMemsetAsync(p->d_iI, 0xff, sizeof(int) * p->batch, g->stream));
        launch_set(p->d_base, 0, g->stream);
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    double bms = 1e30;
    int bmode = g->mode, bby = g->by;
    std::lock_guard<std::mutex> lock(g_table_mu);
    for (int mode : {0, 1, 2, 3})
        for (int by : {1, 2, 4}) {
            if ((mode == 2 && by != 1) || (mode == 3 && by > 2)) continue; /* mode 2: the members' own */
            if (configure(g, mode, by) != SMAT_OK) {
                smat_clear_error();
                continue;
            }
            enqueue_group(g, 0, 1);
            CK(cudaEventRecord(e0, g->stream));
            enqueue_group(g, 0, nsteps);
            CK(cudaEventRecord(e1, g->stream));
            CK(cudaEventSynchronize(e1));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (cudaGetLastError() != cudaSuccess) continue; /* a form whose launches were refused */
            if (ms < bms) {
                bms = ms;
                bmode = mode;
                bby = by;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (size_t i = 0; i < g->m.size(); i++) {
        smat_fdtd_plan *p = g->m[i];
        p->nq = nq[i];
        CK(cudaMemcpyAsync(p->d_iI, p->h_iI.data(), sizeof(int) * p->batch, cudaMemcpyHostToDevice, g->stream));
    }
    CK(cudaStreamSynchronize(g->stream));
    int rc = configure(g, bmode, bby);
    if (rc) return rc;
    drop_group_graph(g);
    if (best) {
        best[0] = bmode;
        best[1] = bby;
    }
    if (best_ms) *best_ms = bms / nsteps;
    return SMAT_OK;
}
