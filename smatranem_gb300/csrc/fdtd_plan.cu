/*
 * Plans: device-resident state of one structure and its batch of excitations,
 * the launch schedule (CUDA-graph captured chunks of steps) and the C ABI of
 * include/smatran_fdtd.h.
 *
 * A plan replaces the reference time loop (FDTDcalc/FDTDsplitfieldMetal.c
 * main :146-167) and its per-step main_calc (:242-329); the host precompute
 * in host_precompute.c replaces main :62-143.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <functional>
#include <memory>
#include <new>
#include <vector>

#include "trace.cuh"
#include "plan_internal.cuh"

using namespace smat;
using namespace smat::plan;

namespace smat {
namespace plan {

Geo make_geo(const smat_fdtd_plan *p)
{
    Geo g;
    g.L0 = p->L[0];
    g.L1 = p->L[1];
    g.L2 = p->L[2];
    g.pl = p->pl;
    g.n3 = p->n3;
    for (int a = 0; a < 3; a++) g.bc[a] = p->iBc[a];
    g.iI = p->iBTIin[2];
    const int m = p->iBTIin[3];
    g.sgn = (double)(m / (m < 0 ? -m : m));
    return g;
}

Dft make_dft(const smat_fdtd_plan *p, bool explicit_phase)
{
    Dft d;
    d.nfreq = p->nfreq;
    d.nq = p->nq;
    for (int i = 0; i < MAX_PLANES; i++) d.planes[i] = p->planes[i];
    d.phase = p->d_phase;
    d.phase32 = p->d_phase32;
    d.xphase = explicit_phase ? p->d_xphase : nullptr;
    d.xphase32 = explicit_phase ? p->d_xphase32 : nullptr;
    d.acc = p->d_acc;
    d.ringK = RING_K;
    d.ring = p->d_ring;
    return d;
}

Src make_src(const smat_fdtd_plan *p, bool explicit_src)
{
    Src s;
    s.base = p->d_base;
    s.sched = p->d_sched;
    s.inc = p->d_inc;
    s.xsrc = explicit_src ? p->d_xsrc : nullptr;
    s.iI = p->d_iI;
    s.sgn = p->d_isgn;
    return s;
}

P64 make_p64(const smat_fdtd_plan *p, bool xp)
{
    P64 q;
    q.g = make_geo(p);
    q.batch = p->batch;
    q.lnotn = p->lnotn;
    q.flags = p->d_flags;
    q.addr = p->d_addr;
    q.cm = p->d_cm;
    q.ca = p->d_ca;
    q.H = p->d_H64;
    q.E = p->d_E64;
    q.Ha = p->d_Ha64;
    q.Ea = p->d_Ea64;
    q.s = make_src(p, xp);
    q.d = make_dft(p, xp);
    return q;
}

P32 make_p32(const smat_fdtd_plan *p, bool xp)
{
    P32 q;
    q.g = make_geo(p);
    q.batch = p->batch;
    q.bh = p->d_bh;
    q.be = p->d_be;
    q.hrec = p->d_hrec;
    q.erec = p->d_erec;
    q.tab = p->d_tab;
    q.pmask = p->d_pmask;
    q.H = p->cur ? p->d_H32b : p->d_H32;
    q.E = p->cur ? p->d_E32b : p->d_E32;
    q.Ha = p->cur ? p->d_Ha32b : p->d_Ha32;
    q.Ea = p->cur ? p->d_Ea32b : p->d_Ea32;
    q.s = make_src(p, xp);
    q.d = make_dft(p, xp);
    return q;
}

/* launch form 6: whole-row tiles of ty rows, z chunks of zc planes */
Row32 make_row(const smat_fdtd_plan *p, bool xp)
{
    Row32 r;
    r.p = make_p32(p, xp);
    r.Hn = p->cur ? p->d_H32 : p->d_H32b;
    r.En = p->cur ? p->d_E32 : p->d_E32b;
    r.Han = p->cur ? p->d_Ha32 : p->d_Ha32b;
    r.Ean = p->cur ? p->d_Ea32 : p->d_Ea32b;
    r.ty = p->ty;
    r.zc = p->zc;
    r.nyt = (p->L[1] + p->ty - 1) / p->ty;
    if (p->zc > 0) {
        r.nzc = (p->L[2] + p->zc - 1) / p->zc;
        r.nitems = p->batch * r.nyt * r.nzc;
        r.ngroups = 0;
    } else {
        /* persistent: as many groups of `batch` CTAs as are resident at once */
        const int resident = sm_count() * (p->max_ctas > 0 ? p->max_ctas : 1);
        r.nzc = 1;
        r.ngroups = resident / p->batch > 0 ? resident / p->batch : 1;
        r.nitems = r.ngroups * p->batch;
    }
    r.qorder = p->d_qorder;
    r.nqp = p->nqp;
    r.has_rec = p->nhgen + p->negen > 0;
    r.worder = p->fused == 6 ? p->ns : 0;
    return r;
}

int sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return 1;
    }
    return n;
}

/* the launches of steps rel0 .. rel0+n-1 relative to *d_base (no bump) */
void enqueue_steps(smat_fdtd_plan *p, int rel0, int n, bool xp)
{
    if (p->precision == SMAT_FP64) {
        const P64 q = make_p64(p, xp);
        for (int i = 0; i < n; i++) {
            launch_h64(q, rel0 + i, p->stream);
            launch_e64(q, rel0 + i, p->stream);
            launch_dft64(q, rel0 + i, p->stream);
        }
    } else if (p->fused == 6) {
        for (int i = 0; i < n; i++) launch_row_step(p, xp, rel0 + i, p->stream);
        launch_flush32(make_p32(p, xp), rel0 + n, n, p->stream);
    } else {
        const P32 q = make_p32(p, xp);
        for (int i = 0; i < n; i++) sweep_step(p, q, rel0 + i, p->stream);
        launch_flush32(q, rel0 + n, n, p->stream);
    }
}

/* One step's update launches of plan p on stream st, without the DFT flush:
 * the plan's own launch form (the whole-row fused step 6, which swaps the
 * field sets, or the sweeps 0 and 2). */
void enqueue_update(smat_fdtd_plan *p, int rel, cudaStream_t st)
{
    if (p->precision != SMAT_FP32) return;
    if (p->fused == 6) {
        launch_row_step(p, false, rel, st);
        return;
    }
    sweep_step(p, make_p32(p, false), rel, st);
}

void launch_row_step(smat_fdtd_plan *p, bool xp, int rel, cudaStream_t st)
{
    const Row32 r = make_row(p, xp);
    launch_row32(r, rel, p->ctas_per_sm, st);
    launch_row_metal(r, rel, p->d_hmetal, p->nhmetal, p->d_emetal, p->nemetal, st);
    p->cur ^= 1;
}

/* One FP32 step as two sweeps (kernels 0 and 2), in z-chunks of szc planes:
 * H on planes [z0, z1), then E on [z0-1, z1-1) -- E of a plane needs H_new of
 * the plane above, H of a plane needs E_old of the plane below, and both
 * still hold at every chunk boundary.  A chunk small enough to stay in L2
 * lets the E sweep read E_old and H_new from L2 rather than HBM. */
void sweep_step(smat_fdtd_plan *p, const P32 &q, int rel, cudaStream_t st)
{
    const int L2 = p->L[2];
    /* a stable-form E cell at z = 0 reads the new H of plane L2-1 through a
     * wrapped z boundary: such plans sweep the whole grid at once */
    const bool whole = p->szc <= 0 || p->szc >= L2 || (p->nstable > 0 && p->iBc[2] != 0);
    const int zc = whole ? L2 : p->szc;
    for (int z0 = 0; z0 < L2; z0 += zc) {
        const int z1 = z0 + zc < L2 ? z0 + zc : L2;
        const int e0 = z0 == 0 ? 0 : z0 - 1, e1 = z1 == L2 ? L2 : z1 - 1;
        if (p->fused == 2) {
            launch_h32v(q, rel, p->by32, p->sweep_mb, z0, z1, p->d_hgen + p->hgen_z[z0],
                        p->hgen_z[z1] - p->hgen_z[z0], st);
            if (e1 > e0)
                launch_e32v(q, rel, p->by32, p->sweep_mb, e0, e1, p->d_egen + p->egen_z[e0],
                            p->egen_z[e1] - p->egen_z[e0], st);
        } else {
            launch_h32(q, rel, p->by32, z0, z1, st);
            if (e1 > e0) launch_e32(q, rel, p->by32, e0, e1, st);
        }
    }
}

void drop_graph(smat_fdtd_plan *p)
{
    if (p->graph) cudaGraphExecDestroy(p->graph);
    p->graph = nullptr;
    p->graph_failed = false;
}

int build_graph(smat_fdtd_plan *p)
{
    if (p->graph || p->graph_failed) return SMAT_OK;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        p->graph_failed = true;
        return SMAT_OK;
    }
    const int cur0 = p->cur;
    enqueue_steps(p, 0, GRAPH_STEPS, false);
    launch_bump(p->d_base, GRAPH_STEPS, p->stream);
    p->cur = cur0;
    cudaError_t e = cudaStreamEndCapture(p->stream, &g);
    if (e != cudaSuccess || !g) {
        cudaGetLastError();
        p->graph_failed = true;
        return SMAT_OK;
    }
    e = cudaGraphInstantiate(&p->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        p->graph = nullptr;
        p->graph_failed = true;
    }
    return SMAT_OK;
}

/* host flags of FP64 cells: class code and "a neighbour has an aux slot" */
void build_flags(const smat_fdtd_plan *p, std::vector<uint8_t> &fl)
{
    const int L0 = p->L[0], L1 = p->L[1], L2 = p->L[2];
    const long long n3 = p->n3;
    fl.assign(n3, 0);
    auto special = [&](long long l) { return p->cont[l] != 'n'; };
    long long l = 0;
    for (int j2 = 0; j2 < L2; j2++)
        for (int j1 = 0; j1 < L1; j1++)
            for (int j0 = 0; j0 < L0; j0++, l++) {
                uint8_t c = CLS_N;
                switch (p->cont[l]) {
                case 'a': c = CLS_A; break;
                case 'h': c = CLS_H; break;
                case 'e': c = CLS_E; break;
                case 'b': c = CLS_B; break;
                default: c = CLS_N;
                }
                const long long xm = l + (j0 == 0 ? L0 - 1 : -1), xp = l + (j0 + 1 == L0 ? -(L0 - 1) : 1);
                const long long sy = L0, sz = (long long)L0 * L1;
                const long long ym = l + (j1 == 0 ? (L1 - 1) * sy : -sy), yp = l + (j1 + 1 == L1 ? -(L1 - 1) * sy : sy);
                const long long zm = l + (j2 == 0 ? (L2 - 1) * sz : -sz), zp = l + (j2 + 1 == L2 ? -(L2 - 1) * sz : sz);
                if (special(xm) || special(ym) || special(zm)) c |= FL_BWD;
                if (special(xp) || special(yp) || special(zp)) c |= FL_FWD;
                fl[l] = c;
            }
}

int check_planes(const smat_fdtd_plan *p, int nq, const int *planes)
{
    for (int q = 0; q < nq; q++) {
        const int z = planes[q];
        if (z < 0 || z >= p->L[2]) return smat_fail(SMAT_EINVAL, "monitor plane %d outside 0..%d", z, p->L[2] - 1);
        for (long long i = 0; i < p->pl; i++)
            if (p->cont[i + (long long)p->pl * z] == 'a')
                return smat_fail(SMAT_EMONITOR, "iBTIin error: monitor plane %d holds a PML cell", z);
    }
    return SMAT_OK;
}

/* (re)allocate DFT accumulators and the FP32 ring for nfreq x nq planes */
int setup_dft(smat_fdtd_plan *p, int nfreq, int nq, const int *planes)
{
    if (nq > MAX_PLANES) return smat_fail(SMAT_EINVAL, "at most %d monitor planes", MAX_PLANES);
    int rc;
    for (int q = 0; q < nq; q++)
        if (planes[q] < 0 || planes[q] >= p->L[2])
            return smat_fail(SMAT_EINVAL, "monitor plane %d outside 0..%d", planes[q], p->L[2] - 1);
    drop_graph(p);
    const size_t acc_n = (size_t)p->batch * nfreq * nq * 4 * p->pl * 2;
    const size_t ring_n = p->precision == SMAT_FP32 ? (size_t)p->batch * RING_K * nq * 4 * p->pl : 0;
    const size_t old_acc = (size_t)p->batch * p->nfreq * p->nq * 4 * p->pl * 2;
    const size_t old_ring = p->precision == SMAT_FP32 ? (size_t)p->batch * RING_K * p->nq * 4 * p->pl : 0;
    if (acc_n != old_acc || !p->d_acc) {
        if (p->d_acc) cudaFree(p->d_acc), p->dev_bytes -= old_acc * 8;
        p->d_acc = nullptr;
        if (acc_n) {
            rc = dalloc(&p->d_acc, acc_n, p->stream);
            if (rc) return rc;
            p->dev_bytes += acc_n * 8;
        }
    }
    if (ring_n != old_ring || (!p->d_ring && ring_n)) {
        if (p->d_ring) cudaFree(p->d_ring), p->dev_bytes -= old_ring * 4;
        p->d_ring = nullptr;
        if (ring_n) {
            rc = dalloc(&p->d_ring, ring_n, p->stream);
            if (rc) return rc;
            p->dev_bytes += ring_n * 4;
        }
    }
    p->nfreq = nfreq;
    p->nq = nq;
    for (int i = 0; i < MAX_PLANES; i++) p->planes[i] = i < nq ? planes[i] : -1;
    if (p->d_acc) CK(cudaMemsetAsync(p->d_acc, 0, acc_n * 8, p->stream));
    return SMAT_OK;
}

int common_alloc(smat_fdtd_plan *p)
{
    int rc;
    if ((rc = p->alloc(&p->d_base, 1))) return rc;
    if ((rc = p->alloc(&p->d_inc, (size_t)p->batch * 8 * p->pl))) return rc;
    if ((rc = p->alloc(&p->d_xsrc, (size_t)4 * p->pl))) return rc;
    if ((rc = p->alloc(&p->d_xphase, 4))) return rc;
    if ((rc = p->alloc(&p->d_xphase32, 8))) return rc;
    if ((rc = p->alloc(&p->d_scratch, 4))) return rc;
    if ((rc = p->alloc(&p->d_iI, p->batch)) || (rc = p->alloc(&p->d_isgn, p->batch))) return rc;
    if ((rc = p->alloc(&p->d_err, 1))) return rc;
    {
        const int m = p->iBTIin[3];
        std::vector<int> ii(p->batch, p->iBTIin[2]);
        p->h_iI = ii;
        std::vector<double> sg(p->batch, (double)(m / (m < 0 ? -m : m)));
        CK(p->cpy(p->d_iI, ii.data(), ii.size() * sizeof(int), cudaMemcpyHostToDevice));
        CK(p->cpy(p->d_isgn, sg.data(), sg.size() * 8, cudaMemcpyHostToDevice));
        CK(cudaStreamSynchronize(p->stream));
    }
    /* the reference DFT: one frequency on planes iB and iT */
    const int pls[2] = {p->iBTIin[0], p->iBTIin[1]};
    rc = setup_dft(p, 1, 2, pls);
    if (rc) return rc;
    p->ref_dft = true;
    p->ref_planes_ok = check_planes(p, 2, pls) == SMAT_OK;
    smat_clear_error();
    return SMAT_OK;
}

int validate_common(const int L[4], const int iBc[3], const int iBTIin[4], int batch)
{
    if (!L || L[0] <= 0 || L[1] <= 0 || L[2] <= 0 || L[3] < 0)
        return smat_fail(SMAT_EINVAL, "L must be positive (got %d %d %d %d)", L ? L[0] : 0, L ? L[1] : 0, L ? L[2] : 0,
                         L ? L[3] : 0);
    if ((long long)L[0] * L[1] * L[2] >= (1LL << 31) / 3)
        return smat_fail(SMAT_EINVAL, "grid too large for 32-bit reference indices");
    if (!iBc || !iBTIin) return smat_fail(SMAT_EINVAL, "iBc and iBTIin are required");
    for (int a = 0; a < 3; a++)
        if (iBc[a] < -1 || iBc[a] > 1) return smat_fail(SMAT_EINVAL, "iBc[%d] = %d not in {-1,0,1}", a, iBc[a]);
    if (iBTIin[3] == 0) return smat_fail(SMAT_EINVAL, "inci_mode = 0!");
    for (int i = 0; i < 3; i++)
        if (iBTIin[i] < 0 || iBTIin[i] >= L[2])
            return smat_fail(SMAT_EINVAL, "plane iBTIin[%d] = %d outside 0..%d", i, iBTIin[i], L[2] - 1);
    if (batch < 1) return smat_fail(SMAT_EINVAL, "batch must be >= 1");
    return SMAT_OK;
}

smat_fdtd_plan *new_plan(const int L[4], const int iBc[3], const int iBTIin[4], int precision, int batch,
                         void *stream)
{
    smat_fdtd_plan *p = new (std::nothrow) smat_fdtd_plan();
    if (!p) return nullptr;
    memcpy(p->L, L, sizeof p->L);
    memcpy(p->iBc, iBc, sizeof p->iBc);
    memcpy(p->iBTIin, iBTIin, sizeof p->iBTIin);
    p->precision = precision;
    p->batch = batch;
    p->n3 = (long long)L[0] * L[1] * L[2];
    p->pl = L[0] * L[1];
    if (stream) {
        p->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete p;
            return nullptr;
        }
        p->own_stream = true;
    }
    return p;
}

/* FP64 device arrays from the reference coefficient arrays (AoS -> SoA) */
int upload_f64(smat_fdtd_plan *p, const double *Ah, const double *Bh, const double *Ae, const double *Be)
{
    int rc;
    const long long n3 = p->n3;
    const int ln = p->lnotn;
    std::vector<uint8_t> fl;
    build_flags(p, fl);
    if ((rc = p->alloc(&p->d_flags, n3))) return rc;
    if ((rc = p->alloc(&p->d_addr, n3))) return rc;
    if ((rc = p->alloc(&p->d_cm, 12 * (size_t)n3))) return rc;
    if ((rc = p->alloc(&p->d_ca, 12 * (size_t)ln))) return rc;
    const size_t fs = (size_t)p->batch * 3 * n3, as = (size_t)p->batch * 3 * (ln + 1);
    if ((rc = p->alloc(&p->d_H64, fs)) || (rc = p->alloc(&p->d_E64, fs))) return rc;
    if ((rc = p->alloc(&p->d_Ha64, as)) || (rc = p->alloc(&p->d_Ea64, as))) return rc;
    std::vector<double> cm(12 * (size_t)n3), ca(12 * (size_t)ln);
    const double *src[4] = {Ah, Bh, Ae, Be};
    for (int w = 0; w < 4; w++)
        for (int c = 0; c < 3; c++) {
            for (long long l = 0; l < n3; l++) cm[((size_t)w * 3 + c) * n3 + l] = src[w][c + 3 * l];
            for (int a = 0; a < ln; a++) ca[((size_t)w * 3 + c) * ln + a] = src[w][c + 3 * (n3 + a)];
        }
    CK(p->cpy(p->d_flags, fl.data(), n3, cudaMemcpyHostToDevice));
    CK(p->cpy(p->d_addr, p->addr.data(), n3 * sizeof(int), cudaMemcpyHostToDevice));
    CK(p->cpy(p->d_cm, cm.data(), cm.size() * 8, cudaMemcpyHostToDevice));
    if (ln) CK(p->cpy(p->d_ca, ca.data(), ca.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaStreamSynchronize(p->stream));
    return SMAT_OK;
}

/* FP32 packed stream: per cell B = 1/(tR Re mu) (A == 1) for ordinary and
 * separable split cells, records for everything else. */
int upload_f32(smat_fdtd_plan *p, const smat_fdtd_desc *d, const double *Ah, const double *Bh, const double *Ae,
               const double *Be)
{
    int rc;
    const long long n3 = p->n3;
    const double iR = d->invtau_R, iI = d->invtau_I;
    const double *mu = d->mu, *ep = d->epsi;
    std::unique_ptr<float[]> bh(new (std::nothrow) float[3 * n3]), be(new (std::nothrow) float[3 * n3]);
    if (!bh || !be) return smat_fail(SMAT_ENOMEM, "create: out of host memory for the packed coefficients");
    auto aux = [&](long long l, int c) { return (size_t)c + 3 * (size_t)(n3 + p->addr[l]); };
    /* The cells go over host worker threads in runs of whole z planes.  Each
     * run numbers its records from 0 in cell order and keeps the cells they
     * belong to; joining the runs in order afterwards gives the numbering of
     * one pass over all cells, so the packed arrays do not depend on the
     * number of threads. */
    struct Run {
        std::vector<Rec32> rec[2]; /* 0: H (mu), 1: E (epsi) */
        std::vector<int> cell[2];
    };
    const int nrun = std::min(host_threads(n3), p->L[2]);
    std::vector<Run> runs(nrun);
    struct PackCtx {
        std::vector<Run> *runs;
        std::function<void(Run &, long long, long long)> pack;
        int nrun, L2;
        long long pl;
    } ctx{&runs, nullptr, nrun, p->L[2], p->pl};
    ctx.pack = [&](Run &run, long long l0, long long l1) {
        for (long long l = l0; l < l1; l++) {
            const char k = p->cont[l];
            const bool pec = d->pec && d->pec[l];
            for (int side = 0; side < 2; side++) {
                float *cf = side ? be.get() : bh.get();
                const double *m = side ? ep : mu;
                const double *A = side ? Ae : Ah, *B = side ? Be : Bh;
                const bool lossless = m[2 * (3 * l + 0) + 1] == 0.0 && m[2 * (3 * l + 1) + 1] == 0.0 &&
                                      m[2 * (3 * l + 2) + 1] == 0.0;
                bool simple = false;
                if (k == 'n')
                    simple = lossless && !(side == 1 && pec) && (float)A[3 * l] == 1.0f &&
                             (float)A[1 + 3 * l] == 1.0f && (float)A[2 + 3 * l] == 1.0f;
                else if (k == 'a')
                    simple = lossless;
                if (simple) {
                    for (int c = 0; c < 3; c++) cf[c * n3 + l] = (float)(1. / (iR * m[2 * (3 * l + c)]));
                    continue;
                }
                /* a record: everything else (a few per mille of the cells) */
                Rec32 r;
                memset(&r, 0, sizeof r);
                for (int c = 0; c < 3; c++) {
                    r.A0[c] = (float)A[c + 3 * l];
                    r.B0[c] = (float)B[c + 3 * l];
                    if (k != 'n') {
                        r.A1[c] = (float)A[aux(l, c)];
                        r.B1[c] = (float)B[aux(l, c)];
                    }
                }
                if (k == 'n') {
                    r.kind = RK_N;
                } else if (k == 'a') {
                    r.kind = RK_A;
                } else {
                    const bool stable_here = side == 0 ? (k == 'h' || k == 'b') : (k == 'e' || k == 'b');
                    r.kind = stable_here ? RK_STABLE : RK_FROZEN;
                }
                if (side == 1 && pec) {
                    for (int c = 0; c < 3; c++) r.A0[c] = r.B0[c] = 0.0f;
                }
                /* the coefficient slot holds NaN, the next one the record number */
                const int idx = (int)run.rec[side].size();
                cf[l] = std::nanf("");
                memcpy(&cf[n3 + l], &idx, 4);
                cf[2 * n3 + l] = 0.0f;
                run.rec[side].push_back(r);
                run.cell[side].push_back((int)l);
            }
        }
    };
    host_parallel_for(
        nrun, nrun,
        [](void *c, long long t0, long long t1) {
            PackCtx &x = *static_cast<PackCtx *>(c);
            for (long long t = t0; t < t1; t++) {
                const long long z0 = x.L2 * t / x.nrun, z1 = x.L2 * (t + 1) / x.nrun;
                x.pack((*x.runs)[t], z0 * x.pl, z1 * x.pl);
            }
        },
        &ctx);
    std::vector<Rec32> hrec, erec;
    std::vector<int> hgen, egen;
    for (const Run &run : runs)
        for (int side = 0; side < 2; side++) {
            std::vector<Rec32> &recs = side ? erec : hrec;
            std::vector<int> &gen = side ? egen : hgen;
            float *cf = side ? be.get() : bh.get();
            const int base = (int)recs.size();
            if (base)
                for (size_t i = 0; i < run.cell[side].size(); i++) {
                    const int idx = base + (int)i;
                    memcpy(&cf[n3 + run.cell[side][i]], &idx, 4);
                }
            recs.insert(recs.end(), run.rec[side].begin(), run.rec[side].end());
            gen.insert(gen.end(), run.cell[side].begin(), run.cell[side].end());
        }
    runs.clear();
    /* 1-D sigma tables: rows A_h, G_h, A_e, G_e over the three axes */
    const int S = p->L[0] + p->L[1] + p->L[2];
    std::vector<float> tab(4 * (size_t)S);
    std::vector<uint8_t> pmask(S);
    const int aoff[3] = {0, p->L[0], p->L[0] + p->L[1]};
    const int soff[3] = {0, 2 * p->L[0], 2 * (p->L[0] + p->L[1])};
    for (int a = 0; a < 3; a++)
        for (int j = 0; j < p->L[a]; j++) {
            const double sh = d->sigma[soff[a] + 2 * j], se = d->sigma[soff[a] + 1 + 2 * j];
            tab[0 * S + aoff[a] + j] = (float)((iR - iI * sh) / (iR + iI * sh));
            tab[1 * S + aoff[a] + j] = (float)(iR / (iR + iI * sh));
            tab[2 * S + aoff[a] + j] = (float)((iR - iI * se) / (iR + iI * se));
            tab[3 * S + aoff[a] + j] = (float)(iR / (iR + iI * se));
            pmask[aoff[a] + j] = std::fabs(sh) > 10.0 * 2.220446049250313e-16 || std::fabs(se) > 10.0 * 2.220446049250313e-16;
        }
    if ((rc = p->alloc(&p->d_bh, 3 * (size_t)n3)) || (rc = p->alloc(&p->d_be, 3 * (size_t)n3))) return rc;
    if ((rc = p->alloc(&p->d_tab, 4 * (size_t)S)) || (rc = p->alloc(&p->d_pmask, (size_t)S))) return rc;
    if ((rc = p->alloc(&p->d_hrec, hrec.size() + 1)) || (rc = p->alloc(&p->d_erec, erec.size() + 1))) return rc;
    const size_t fs = (size_t)p->batch * 3 * n3;
    if ((rc = p->alloc(&p->d_H32, fs)) || (rc = p->alloc(&p->d_E32, fs))) return rc;
    if ((rc = p->alloc(&p->d_Ha32, fs)) || (rc = p->alloc(&p->d_Ea32, fs))) return rc;
    if ((rc = p->alloc(&p->d_H32b, fs)) || (rc = p->alloc(&p->d_E32b, fs))) return rc;
    if ((rc = p->alloc(&p->d_Ha32b, fs)) || (rc = p->alloc(&p->d_Ea32b, fs))) return rc;
    p->nstable = 0;
    for (const Rec32 &r : erec) p->nstable += r.kind == RK_STABLE;
    p->nhgen = (int)hgen.size();
    p->negen = (int)egen.size();
    p->hgen_host = hgen;
    p->egen_host = egen;
    p->hgen_z.assign(p->L[2] + 1, 0);
    p->egen_z.assign(p->L[2] + 1, 0);
    for (int z = 0; z <= p->L[2]; z++) {
        const long long first = (long long)z * p->pl;
        p->hgen_z[z] = (int)(std::lower_bound(hgen.begin(), hgen.end(), first) - hgen.begin());
        p->egen_z[z] = (int)(std::lower_bound(egen.begin(), egen.end(), first) - egen.begin());
    }
    if ((rc = p->alloc(&p->d_hgen, hgen.size() + 1)) || (rc = p->alloc(&p->d_egen, egen.size() + 1))) return rc;
    if (!hgen.empty())
        CK(p->cpy(p->d_hgen, hgen.data(), hgen.size() * sizeof(int), cudaMemcpyHostToDevice));
    if (!egen.empty())
        CK(p->cpy(p->d_egen, egen.data(), egen.size() * sizeof(int), cudaMemcpyHostToDevice));
    /* record kinds; the cells of metal records (stable-form or frozen
     * components), which kernel 6 finishes in a second launch */
    std::vector<int> metal[2];
    for (int side = 0; side < 2; side++) {
        const std::vector<Rec32> &recs = side ? erec : hrec;
        const std::vector<int> &gen = side ? egen : hgen;
        for (size_t i = 0; i < recs.size(); i++) {
            const int kind = recs[i].kind;
            if (kind == RK_STABLE || kind == RK_FROZEN) {
                p->nrec_metal++;
                metal[side].push_back(gen[i]);
            }
            if (kind == RK_A) p->nrec_split++;
        }
    }
    p->nhmetal = (int)metal[0].size();
    p->nemetal = (int)metal[1].size();
    if ((rc = p->alloc(&p->d_hmetal, metal[0].size() + 1)) || (rc = p->alloc(&p->d_emetal, metal[1].size() + 1)))
        return rc;
    if (!metal[0].empty())
        CK(p->cpy(p->d_hmetal, metal[0].data(), metal[0].size() * sizeof(int), cudaMemcpyHostToDevice));
    if (!metal[1].empty())
        CK(p->cpy(p->d_emetal, metal[1].data(), metal[1].size() * sizeof(int), cudaMemcpyHostToDevice));
    if (p->L[0] % 4 == 0) {
        p->fused = 2; /* default: vectorised sweeps where they apply */
        p->by32 = 2;
        /* kernel 6 thread order: quads with a split-PML x index first */
        const int nq = p->L[0] / 4;
        std::vector<int> qorder;
        for (int pass = 0; pass < 2; pass++)
            for (int q = 0; q < nq; q++) {
                const bool px = pmask[4 * q] | pmask[4 * q + 1] | pmask[4 * q + 2] | pmask[4 * q + 3];
                if (px == (pass == 0)) qorder.push_back(q);
                if (pass == 0 && px) p->nqp++;
            }
        if ((rc = p->alloc(&p->d_qorder, (size_t)nq))) return rc;
        CK(p->cpy(p->d_qorder, qorder.data(), nq * sizeof(int), cudaMemcpyHostToDevice));
    }
    CK(p->cpy(p->d_bh, bh.get(), 3 * (size_t)n3 * 4, cudaMemcpyHostToDevice));
    CK(p->cpy(p->d_be, be.get(), 3 * (size_t)n3 * 4, cudaMemcpyHostToDevice));
    CK(p->cpy(p->d_tab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
    CK(p->cpy(p->d_pmask, pmask.data(), pmask.size(), cudaMemcpyHostToDevice));
    if (!hrec.empty())
        CK(p->cpy(p->d_hrec, hrec.data(), hrec.size() * sizeof(Rec32), cudaMemcpyHostToDevice));
    if (!erec.empty())
        CK(p->cpy(p->d_erec, erec.data(), erec.size() * sizeof(Rec32), cudaMemcpyHostToDevice));
    CK(cudaStreamSynchronize(p->stream));
    return SMAT_OK;
}

int finish_create(smat_fdtd_plan *p, int rc, smat_fdtd_plan **out)
{
    if (rc == SMAT_OK) rc = common_alloc(p);
    if (rc == SMAT_OK) {
        cudaError_t e = cudaStreamSynchronize(p->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "plan upload");
    }
    if (rc != SMAT_OK) {
        smat_fdtd_destroy(p);
        return rc;
    }
    *out = p;
    return SMAT_OK;
}

} // namespace plan
} // namespace smat

/* ===================================================================== */

extern "C" int smat_fdtd_create(const smat_fdtd_desc *d, void *stream, smat_fdtd_plan **out)
{
    smat::TraceRange trace_("smat_fdtd_create");
    smat_clear_error();
    if (!d || !out || !d->mu || !d->epsi || !d->sigma) return smat_fail(SMAT_EINVAL, "create: null argument");
    *out = nullptr;
    int rc = validate_common(d->L, d->iBc, d->iBTIin, d->batch);
    if (rc) return rc;
    if (d->precision != SMAT_FP64 && d->precision != SMAT_FP32)
        return smat_fail(SMAT_EINVAL, "precision must be SMAT_FP64 or SMAT_FP32");
    if (!(d->invtau_R > 0) || !std::isfinite(d->invtau_I))
        return smat_fail(SMAT_EINVAL, "invtau_R must be positive and invtau_I finite");
    smat_fdtd_plan *p = new_plan(d->L, d->iBc, d->iBTIin, d->precision, d->batch, stream);
    if (!p) return smat_fail(SMAT_ENOMEM, "plan allocation or stream creation failed");
    p->invtau_R = d->invtau_R;
    p->invtau_I = d->invtau_I;
    const long long n3 = p->n3;
    p->cont.resize(n3);
    p->addr.resize(n3);
    rc = smat_set_address(d->L, d->sigma, d->mu, d->epsi, p->cont.data(), &p->lnotn, p->addr.data());
    if (rc) {
        smat_fdtd_destroy(p);
        return rc;
    }
    if (d->pec)
        for (long long l = 0; l < n3; l++)
            if (d->pec[l] && p->cont[l] != 'n') {
                smat_fdtd_destroy(p);
                return smat_fail(SMAT_EINVAL, "PEC cell %lld is not an ordinary ('n') cell", l);
            }
    /* smat_coefficients fills every entry (its zero fill runs on the host
     * worker threads, which also takes the first touch of the pages off the
     * calling thread), so the arrays start uninitialised */
    const size_t nc = 3 * (size_t)(n3 + p->lnotn);
    std::unique_ptr<double[]> Ah(new (std::nothrow) double[nc]), Bh(new (std::nothrow) double[nc]),
        Ae(new (std::nothrow) double[nc]), Be(new (std::nothrow) double[nc]);
    if (!Ah || !Bh || !Ae || !Be) {
        smat_fdtd_destroy(p);
        return smat_fail(SMAT_ENOMEM, "create: out of host memory for the coefficients");
    }
    rc = smat_coefficients(d->L, p->lnotn, d->sigma, d->mu, d->epsi, p->cont.data(), p->addr.data(), d->invtau_R,
                           d->invtau_I, Ah.get(), Bh.get(), Ae.get(), Be.get());
    if (rc) {
        smat_fdtd_destroy(p);
        return rc;
    }
    if (d->pec)
        for (long long l = 0; l < n3; l++)
            if (d->pec[l])
                for (int c = 0; c < 3; c++) Ae[c + 3 * l] = Be[c + 3 * l] = 0.0;
    rc = p->precision == SMAT_FP64 ? upload_f64(p, Ah.get(), Bh.get(), Ae.get(), Be.get())
                                   : upload_f32(p, d, Ah.get(), Bh.get(), Ae.get(), Be.get());
    return finish_create(p, rc, out);
}

extern "C" int smat_fdtd_create_from_coeffs(const int L[4], const double *Ah, const double *Bh, const double *Ae,
                                            const double *Be, const int iBc[3], const char *Cont,
                                            const int *address_notn, int Lnotn, const int iBTIin[4], int batch,
                                            void *stream, smat_fdtd_plan **out)
{
    smat_clear_error();
    if (!out || !Ah || !Bh || !Ae || !Be || !Cont || !address_notn)
        return smat_fail(SMAT_EINVAL, "create_from_coeffs: null argument");
    *out = nullptr;
    int rc = validate_common(L, iBc, iBTIin, batch);
    if (rc) return rc;
    smat_fdtd_plan *p = new_plan(L, iBc, iBTIin, SMAT_FP64, batch, stream);
    if (!p) return smat_fail(SMAT_ENOMEM, "plan allocation or stream creation failed");
    const long long n3 = p->n3;
    p->cont.assign(Cont, Cont + n3);
    p->addr.assign(address_notn, address_notn + n3);
    p->lnotn = Lnotn;
    int count = 0;
    for (long long l = 0; l < n3; l++) {
        const char k = Cont[l];
        if (k != 'n' && k != 'a' && k != 'h' && k != 'e' && k != 'b') {
            smat_fdtd_destroy(p);
            return smat_fail(SMAT_EINVAL, "Cont[%lld] = %d is not a cell class", l, (int)k);
        }
        const int a = address_notn[l];
        if (k == 'n' ? a != Lnotn : (a < 0 || a >= Lnotn)) {
            smat_fdtd_destroy(p);
            return smat_fail(SMAT_EINVAL, "address_notn[%lld] = %d inconsistent with Cont/Lnotn", l, a);
        }
        count += k != 'n';
    }
    if (count != Lnotn) {
        smat_fdtd_destroy(p);
        return smat_fail(SMAT_EINVAL, "Lnotn = %d but %d non-'n' cells", Lnotn, count);
    }
    rc = upload_f64(p, Ah, Bh, Ae, Be);
    return finish_create(p, rc, out);
}

extern "C" int smat_fdtd_destroy(smat_fdtd_plan *p)
{
    if (!p) return SMAT_OK;
    if (p->stream) cudaStreamSynchronize(p->stream);
    drop_graph(p);
    for (void *a : p->allocations) cudaFree(a);
    if (p->d_acc) cudaFree(p->d_acc);
    if (p->d_ring) cudaFree(p->d_ring);
    if (p->d_sched) cudaFree(p->d_sched);
    if (p->d_phase) cudaFree(p->d_phase);
    if (p->d_phase32) cudaFree(p->d_phase32);
    if (p->own_stream && p->stream) cudaStreamDestroy(p->stream);
    delete p;
    return SMAT_OK;
}

extern "C" int smat_fdtd_info(const smat_fdtd_plan *p, int L[4], int *Lnotn, int *precision, int *batch)
{
    if (!p) return smat_fail(SMAT_EINVAL, "null plan");
    if (L) memcpy(L, p->L, sizeof p->L);
    if (Lnotn) *Lnotn = p->lnotn;
    if (precision) *precision = p->precision;
    if (batch) *batch = p->batch;
    return SMAT_OK;
}

extern "C" long long smat_fdtd_device_bytes(const smat_fdtd_plan *p) { return p ? p->dev_bytes : 0; }

extern "C" int smat_fdtd_set_fields(smat_fdtd_plan *p, int b, const double *H_t, const double *E_t)
{
    smat_clear_error();
    if (!p || !H_t || !E_t || b < 0 || b >= p->batch) return smat_fail(SMAT_EINVAL, "set_fields: bad arguments");
    const long long n3 = p->n3;
    const int ln = p->lnotn;
    for (int w = 0; w < 2; w++) {
        const double *src = w ? E_t : H_t;
        if (p->precision == SMAT_FP64) {
            std::vector<double> m(3 * n3), a(3 * (size_t)(ln + 1), 0.0);
            for (int c = 0; c < 3; c++) {
                for (long long l = 0; l < n3; l++) m[c * n3 + l] = src[c + 3 * l];
                for (int x = 0; x <= ln; x++) a[(size_t)c * (ln + 1) + x] = src[c + 3 * (n3 + x)];
            }
            double *dm = (w ? p->d_E64 : p->d_H64) + (size_t)b * 3 * n3;
            double *da = (w ? p->d_Ea64 : p->d_Ha64) + (size_t)b * 3 * (ln + 1);
            CK(p->cpy(dm, m.data(), m.size() * 8, cudaMemcpyHostToDevice));
            CK(p->cpy(da, a.data(), a.size() * 8, cudaMemcpyHostToDevice));
            CK(cudaStreamSynchronize(p->stream));
        } else {
            std::vector<float> t(3 * n3), a(3 * n3, 0.0f);
            for (int c = 0; c < 3; c++)
                for (long long l = 0; l < n3; l++) {
                    double main = src[c + 3 * l], ax = 0.0;
                    if (p->cont[l] != 'n') ax = src[c + 3 * (n3 + p->addr[l])];
                    t[c * n3 + l] = (float)(main + ax);
                    a[c * n3 + l] = (float)ax;
                }
            const P32 q = make_p32(p, false);
            float *dt = (w ? q.E : q.H) + (size_t)b * 3 * n3;
            float *da = (w ? q.Ea : q.Ha) + (size_t)b * 3 * n3;
            CK(p->cpy(dt, t.data(), t.size() * 4, cudaMemcpyHostToDevice));
            CK(p->cpy(da, a.data(), a.size() * 4, cudaMemcpyHostToDevice));
            CK(cudaStreamSynchronize(p->stream));
        }
    }
    return SMAT_OK;
}

extern "C" int smat_fdtd_get_fields(smat_fdtd_plan *p, int b, double *H_t, double *E_t)
{
    smat_clear_error();
    if (!p || b < 0 || b >= p->batch) return smat_fail(SMAT_EINVAL, "get_fields: bad arguments");
    const long long n3 = p->n3;
    const int ln = p->lnotn;
    for (int w = 0; w < 2; w++) {
        double *dst = w ? E_t : H_t;
        if (!dst) continue;
        if (p->precision == SMAT_FP64) {
            std::vector<double> m(3 * n3), a(3 * (size_t)(ln + 1));
            const double *dm = (w ? p->d_E64 : p->d_H64) + (size_t)b * 3 * n3;
            const double *da = (w ? p->d_Ea64 : p->d_Ha64) + (size_t)b * 3 * (ln + 1);
            CK(p->cpy(m.data(), dm, m.size() * 8, cudaMemcpyDeviceToHost));
            CK(p->cpy(a.data(), da, a.size() * 8, cudaMemcpyDeviceToHost));
            CK(cudaStreamSynchronize(p->stream));
            for (int c = 0; c < 3; c++) {
                for (long long l = 0; l < n3; l++) dst[c + 3 * l] = m[c * n3 + l];
                for (int x = 0; x <= ln; x++) dst[c + 3 * (n3 + x)] = a[(size_t)c * (ln + 1) + x];
            }
        } else {
            std::vector<float> t(3 * n3), a(3 * n3);
            const P32 q = make_p32(p, false);
            const float *dt = (w ? q.E : q.H) + (size_t)b * 3 * n3;
            const float *da = (w ? q.Ea : q.Ha) + (size_t)b * 3 * n3;
            CK(p->cpy(t.data(), dt, t.size() * 4, cudaMemcpyDeviceToHost));
            CK(p->cpy(a.data(), da, a.size() * 4, cudaMemcpyDeviceToHost));
            CK(cudaStreamSynchronize(p->stream));
            memset(dst, 0, sizeof(double) * 3 * (size_t)(n3 + ln + 1));
            for (int c = 0; c < 3; c++)
                for (long long l = 0; l < n3; l++) {
                    if (p->cont[l] == 'n') {
                        dst[c + 3 * l] = t[c * n3 + l];
                    } else {
                        const float ax = a[c * n3 + l];
                        dst[c + 3 * l] = (double)(t[c * n3 + l] - ax);
                        dst[c + 3 * (n3 + p->addr[l])] = ax;
                    }
                }
        }
    }
    return SMAT_OK;
}

extern "C" int smat_fdtd_set_incident(smat_fdtd_plan *p, int b, const double *Hinc, const double *Einc)
{
    smat_clear_error();
    if (!p || !Hinc || !Einc || b < 0 || b >= p->batch) return smat_fail(SMAT_EINVAL, "set_incident: bad arguments");
    const size_t n = 4 * (size_t)p->pl;
    CK(p->cpy(p->d_inc + (size_t)b * 8 * p->pl, Hinc, n * 8, cudaMemcpyHostToDevice));
    CK(p->cpy(p->d_inc + (size_t)b * 8 * p->pl + n, Einc, n * 8, cudaMemcpyHostToDevice));
    CK(cudaStreamSynchronize(p->stream));
    return SMAT_OK;
}

extern "C" int smat_fdtd_set_source_plane(smat_fdtd_plan *p, int b, int iI, int inci_mode)
{
    smat_clear_error();
    if (!p || b < 0 || b >= p->batch || iI < 0 || iI >= p->L[2] || inci_mode == 0)
        return smat_fail(SMAT_EINVAL, "set_source_plane: bad arguments");
    const double sg = (double)(inci_mode / (inci_mode < 0 ? -inci_mode : inci_mode));
    p->h_iI[b] = iI;
    CK(p->cpy(p->d_iI + b, &iI, sizeof(int), cudaMemcpyHostToDevice));
    CK(p->cpy(p->d_isgn + b, &sg, 8, cudaMemcpyHostToDevice));
    CK(cudaStreamSynchronize(p->stream));
    return SMAT_OK;
}

extern "C" int smat_fdtd_set_schedule(smat_fdtd_plan *p, int nsteps, const double *src, int nfreq, int nplanes,
                                      const int *planes, const double *phase)
{
    smat_clear_error();
    if (!p || nsteps <= 0 || !src || nfreq < 0 || (nfreq > 0 && (!phase || !planes || nplanes <= 0)))
        return smat_fail(SMAT_EINVAL, "set_schedule: bad arguments");
    int rc = setup_dft(p, nfreq, nfreq > 0 ? nplanes : 0, planes);
    if (rc) return rc;
    p->ref_dft = false;
    if (p->d_sched) cudaFree(p->d_sched), p->d_sched = nullptr;
    if (p->d_phase) cudaFree(p->d_phase), p->d_phase = nullptr;
    if (p->d_phase32) cudaFree(p->d_phase32), p->d_phase32 = nullptr;
    if ((rc = dalloc(&p->d_sched, 6 * (size_t)nsteps, p->stream))) return rc;
    CK(p->cpy(p->d_sched, src, 6 * (size_t)nsteps * 8, cudaMemcpyHostToDevice));
    if (nfreq > 0) {
        const size_t np = 4 * (size_t)nsteps * nfreq;
        if ((rc = dalloc(&p->d_phase, np, p->stream))) return rc;
        CK(p->cpy(p->d_phase, phase, np * 8, cudaMemcpyHostToDevice));
        if (p->precision == SMAT_FP32) {
            /* the FP32 flush's phase pairs: per step and frequency, for H then
             * E, {hi re, hi im, lo re, lo im} with hi = fl(phase), lo =
             * fl(phase - hi) */
            std::vector<float> ph32(2 * np);
            for (size_t i = 0; i < np / 4; i++)
                for (int h = 0; h < 2; h++)
                    for (int c = 0; c < 2; c++) {
                        const double v = phase[4 * i + 2 * h + c];
                        const float hi = (float)v;
                        ph32[8 * i + 4 * h + c] = hi;
                        ph32[8 * i + 4 * h + 2 + c] = (float)(v - (double)hi);
                    }
            if ((rc = dalloc(&p->d_phase32, 2 * np, p->stream))) return rc;
            CK(p->cpy(p->d_phase32, ph32.data(), 2 * np * 4, cudaMemcpyHostToDevice));
        }
    }
    p->nsched = nsteps;
    CK(cudaStreamSynchronize(p->stream));
    return SMAT_OK;
}

extern "C" int smat_cw_schedule(int N_2pi, const int tp[3], double *src, double *phase)
{
    smat_clear_error();
    if (N_2pi <= 0 || !tp || tp[0] < 0 || tp[1] < 0 || tp[2] <= 0 || !src || !phase)
        return smat_fail(SMAT_EINVAL, "cw_schedule: bad arguments");
    return host_cw_schedule(N_2pi, tp, src, phase);
}

extern "C" int smat_fdtd_set_cw_schedule(smat_fdtd_plan *p, int N_2pi, const int tp[3])
{
    smat_clear_error();
    if (!p || N_2pi <= 0 || !tp || tp[0] < 0 || tp[1] < 0 || tp[2] <= 0)
        return smat_fail(SMAT_EINVAL, "set_cw_schedule: bad arguments");
    if (!p->ref_planes_ok) {
        const int pls[2] = {p->iBTIin[0], p->iBTIin[1]};
        return check_planes(p, 2, pls);
    }
    const int nsteps = tp[2] * N_2pi;
    std::vector<double> src(6 * (size_t)nsteps), ph(4 * (size_t)nsteps);
    int rc = host_cw_schedule(N_2pi, tp, src.data(), ph.data());
    if (rc) return rc;
    const int planes[2] = {p->iBTIin[0], p->iBTIin[1]};
    rc = smat_fdtd_set_schedule(p, nsteps, src.data(), 1, 2, planes, ph.data());
    if (rc) return rc;
    p->ref_dft = true;
    return SMAT_OK;
}

extern "C" int smat_fdtd_step(smat_fdtd_plan *p, const double *Hi, const double *Ei, const double *ExpN2)
{
    smat_clear_error();
    if (!p || !Hi || !Ei || !ExpN2) return smat_fail(SMAT_EINVAL, "step: bad arguments");
    if (!p->ref_dft || p->nfreq < 1) return smat_fail(SMAT_ESTATE, "step: the reference DFT is not configured");
    if (!p->ref_planes_ok) {
        const int pls[2] = {p->iBTIin[0], p->iBTIin[1]};
        return check_planes(p, 2, pls);
    }
    const int nf = p->nfreq;
    p->nfreq = 1; /* explicit phases drive frequency slot 0 only */
    const size_t n = 2 * (size_t)p->pl;
    float x32[8]; /* the phase pairs of the FP32 flush: H then E, {hi re, hi im, lo re, lo im} */
    for (int h = 0; h < 2; h++)
        for (int c = 0; c < 2; c++) {
            const float hi = (float)ExpN2[2 * h + c];
            x32[4 * h + c] = hi;
            x32[4 * h + 2 + c] = (float)(ExpN2[2 * h + c] - (double)hi);
        }
    cudaError_t e = p->cpy(p->d_xsrc, Hi, n * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = p->cpy(p->d_xsrc + n, Ei, n * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = p->cpy(p->d_xphase, ExpN2, 4 * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = p->cpy(p->d_xphase32, x32, 8 * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        launch_set(p->d_base, 0, p->stream);
        enqueue_steps(p, 0, 1, true);
        e = cudaStreamSynchronize(p->stream);
    }
    p->nfreq = nf;
    if (e != cudaSuccess) return cuda_fail(e, "step");
    return SMAT_OK;
}

extern "C" int smat_fdtd_run(smat_fdtd_plan *p, int k_begin, int k_end)
{
    smat::TraceRange trace_("smat_fdtd_run");
    smat_clear_error();
    if (!p || k_begin < 0 || k_end < k_begin) return smat_fail(SMAT_EINVAL, "run: bad step range");
    if (!p->d_sched) return smat_fail(SMAT_ESTATE, "run: no schedule (call set_cw_schedule or set_schedule)");
    if (k_end > p->nsched) return smat_fail(SMAT_EINVAL, "run: k_end %d beyond the %d-step schedule", k_end, p->nsched);
    launch_set(p->d_base, k_begin, p->stream);
    int n = k_end - k_begin;
    if (p->precision == SMAT_FP32 && p->fused == 6 && p->cur != 0 && n >= GRAPH_STEPS + 1) {
        /* graphs are captured from field set 0: take one step to get there */
        enqueue_steps(p, 0, 1, false);
        launch_bump(p->d_base, 1, p->stream);
        n -= 1;
    }
    if (n >= GRAPH_STEPS) build_graph(p);
    while (n >= GRAPH_STEPS) {
        if (p->graph) {
            CK(cudaGraphLaunch(p->graph, p->stream));
            /* the captured chunk toggled cur an even number of times */
        } else {
            enqueue_steps(p, 0, GRAPH_STEPS, false);
            launch_bump(p->d_base, GRAPH_STEPS, p->stream);
        }
        n -= GRAPH_STEPS;
    }
    if (n > 0) {
        enqueue_steps(p, 0, n, false);
        launch_bump(p->d_base, n, p->stream);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "run: launch");
    return SMAT_OK;
}

extern "C" int smat_fdtd_time_kernels(smat_fdtd_plan *p, int k_begin, int nsteps, double *ms)
{
    smat_clear_error();
    if (!p || !ms || nsteps <= 0 || k_begin < 0 || k_begin + nsteps > p->nsched)
        return smat_fail(SMAT_EINVAL, "time_kernels: bad arguments");
    cudaEvent_t ev[4];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    double acc[3] = {0, 0, 0};
    float t;
    launch_set(p->d_base, k_begin, p->stream);
    const P64 q64 = make_p64(p, false);
    for (int i = 0; i < nsteps; i++) {
        const P32 q32 = make_p32(p, false);
        CK(cudaEventRecord(ev[0], p->stream));
        if (p->precision == SMAT_FP64) launch_h64(q64, i, p->stream);
        else if (p->fused == 6) {
            launch_row_step(p, false, i, p->stream);
        } else if (p->szc > 0 && p->szc < p->L[2]) {
            sweep_step(p, q32, i, p->stream); /* chunked sweeps: the whole step in ms[0] */
        } else if (p->fused == 2) {
            launch_h32v(q32, i, p->by32, p->sweep_mb, 0, p->L[2], p->d_hgen, p->nhgen, p->stream);
        } else {
            launch_h32(q32, i, p->by32, 0, p->L[2], p->stream);
        }
        CK(cudaEventRecord(ev[1], p->stream));
        if (p->precision == SMAT_FP64) launch_e64(q64, i, p->stream);
        else if (p->fused == 6 || (p->szc > 0 && p->szc < p->L[2])) {
        } else if (p->fused == 2)
            launch_e32v(q32, i, p->by32, p->sweep_mb, 0, p->L[2], p->d_egen, p->negen, p->stream);
        else if (p->fused == 0) launch_e32(q32, i, p->by32, 0, p->L[2], p->stream);
        CK(cudaEventRecord(ev[2], p->stream));
        if (p->precision == SMAT_FP64) launch_dft64(q64, i, p->stream);
        else if ((i + 1) % RING_K == 0 || i + 1 == nsteps) {
            const int cnt = (i + 1) % RING_K == 0 ? RING_K : (i + 1) % RING_K;
            launch_flush32(make_p32(p, false), i + 1, cnt, p->stream);
        }
        CK(cudaEventRecord(ev[3], p->stream));
        CK(cudaEventSynchronize(ev[3]));
        for (int k = 0; k < 3; k++) {
            CK(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
            acc[k] += t;
        }
    }
    launch_bump(p->d_base, nsteps, p->stream);
    CK(cudaStreamSynchronize(p->stream));
    for (auto &e : ev) cudaEventDestroy(e);
    ms[0] = acc[0] / nsteps;
    ms[1] = acc[1] / nsteps;
    ms[2] = acc[2] / nsteps;
    return SMAT_OK;
}

extern "C" int smat_fdtd_set_tuning(smat_fdtd_plan *p, int fused, int tile_y, int z_chunk, int ctas_per_sm,
                                    int slots)
{
    smat_clear_error();
    if (!p) return smat_fail(SMAT_EINVAL, "null plan");
    if (fused != 0 && fused != 2 && fused != 6)
        return smat_fail(SMAT_EINVAL, "set_tuning: kernel 0 (sweeps), 2 (vector sweeps) or 6 (fused step, whole "
                                      "rows)");
    if (fused == 6) {
        /* whole-row fused step: tile_y rows per CTA, z chunks, ctas_per_sm = register bound 1..3 */
        if (p->L[0] % 4 != 0) return smat_fail(SMAT_EINVAL, "set_tuning: kernel 6 needs L0 %% 4 == 0");
        if (tile_y < 1 || tile_y > 16 || z_chunk < 0 || ctas_per_sm < 1 || ctas_per_sm > 3 || slots < 0 || slots > 1)
            return smat_fail(SMAT_EINVAL, "set_tuning: kernel 6 takes tile_y in 1..16, z_chunk >= 0 (0: persistent "
                                          "CTAs), ctas_per_sm (register bound) 1..3 and slots (warp order) 0 or 1");
        const int zc = z_chunk == 0 || z_chunk >= p->L[2] ? (z_chunk == 0 ? 0 : p->L[2]) : z_chunk;
        const int occ =
            row32_max_ctas_per_sm(p->L[0], tile_y, ctas_per_sm, zc > 0 ? zc : p->L[2], p->nhgen + p->negen > 0);
        if (occ < 1)
            return smat_fail(SMAT_EINVAL, "set_tuning: kernel 6 with %d rows of %d cells does not fit an SM at %d "
                                          "CTAs per SM", tile_y, p->L[0], ctas_per_sm);
        p->ty = tile_y;
        p->zc = zc;
        p->ctas_per_sm = ctas_per_sm;
        p->max_ctas = occ;
        p->ns = slots; /* kernel 6: the warp order */
        p->fused = 6;
        drop_graph(p);
        return SMAT_OK;
    }
    if (fused == 2 && (p->L[0] % 4 != 0 || tile_y < 1 || tile_y > 4))
        return smat_fail(SMAT_EINVAL, "set_tuning: vector sweeps need L0 %% 4 == 0 and tile_y in 1..4");
    if (tile_y < 1 || tile_y > 8) return smat_fail(SMAT_EINVAL, "set_tuning: block_y in 1..8");
    if (z_chunk < 0) return smat_fail(SMAT_EINVAL, "set_tuning: z_chunk >= 0 (0: whole grid per sweep)");
    if (ctas_per_sm != 0 && ctas_per_sm != 5 && ctas_per_sm != 6 && ctas_per_sm != 8 &&
        !(fused == 2 && ctas_per_sm == -3))
        return smat_fail(SMAT_EINVAL, "set_tuning: sweeps take ctas_per_sm 0 (= 5), 5, 6 or 8 (register bound), "
                                      "or -3 (vector sweeps, two planes per thread)");
    p->by32 = tile_y;
    p->szc = z_chunk >= p->L[2] ? 0 : z_chunk;
    p->sweep_mb = ctas_per_sm == 0 ? 5 : ctas_per_sm;
    p->fused = fused;
    drop_graph(p);
    return SMAT_OK;
}

/* Times each candidate launch configuration over nsteps steps and keeps the
 * fastest.  Runs on the zero state with sources and DFT sampling switched off,
 * so a plan whose fields are all zero is left exactly as it was. */
extern "C" int smat_fdtd_autotune(smat_fdtd_plan *p, int nsteps, int best[5], double *best_ms)
{
    smat::TraceRange trace_("smat_fdtd_autotune");
    smat_clear_error();
    if (!p || nsteps < 1) return smat_fail(SMAT_EINVAL, "autotune: bad arguments");
    if (p->precision != SMAT_FP32) {
        if (best) smat_fdtd_get_tuning(p, best);
        if (best_ms) *best_ms = 0;
        return SMAT_OK;
    }
    int finite = 0;
    double mx = 0;
    int rc = smat_fdtd_check_finite(p, &finite, &mx);
    if (rc) return rc;
    if (mx != 0.0) return smat_fail(SMAT_ESTATE, "autotune: needs the zero state (call it before set_fields/run)");
    struct Cand {
        int fused, ty, zc, ctas, ns;
    };
    std::vector<Cand> cands;
    const int L2 = p->L[2];
    /* sweeps, whole grid or z-chunked (chunk sizes that leave L2 a useful share) */
    const int chunks[] = {0, 2, 4, 8, 16};
    if (p->L[0] % 4 == 0) {
        for (int by : {1, 2})
            for (int mb : {5, 6, -3}) cands.push_back({2, by, 0, mb, 4});
        for (int by : {1, 2})
            for (int zc : chunks)
                if (zc > 0 && zc < L2) cands.push_back({2, by, zc, 5, 4});
        cands.push_back({2, 4, 0, 5, 4});
    }
    /* whole-row fused step, the halo row's warps beside the split quads'
     * (warp order 1: 0.5 % faster on the 256x192x160 bend, 5-row tiles) */
    if (p->L[0] % 4 == 0)
        for (int ty : {1, 2, 4, 5})
            for (int mb : {1, 2})
                for (int zc : {0, L2, 40, 32, 24, 20})
                    if (zc <= L2 && !(zc < 48 && zc >= L2)) cands.push_back({6, ty, zc, mb, 1});
    cands.push_back({0, 4, 0, 0, 4});
    cands.push_back({0, 8, 0, 0, 4});
    cands.push_back({0, 4, 4 < L2 ? 4 : 0, 0, 4});
    const int nq = p->nq;
    p->nq = 0;
    CK(cudaMemsetAsync(p->d_iI, 0xff, sizeof(int) * p->batch, p->stream));
    int save[5];
    smat_fdtd_get_tuning(p, save);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    double bms = 1e30;
    /* SMATRAN_AUTOTUNE_VERBOSE=1 prints every candidate's time to stderr */
    const char *vs = getenv("SMATRAN_AUTOTUNE_VERBOSE");
    const bool verbose = vs && vs[0] && vs[0] != '0';
    Cand bc = {save[0], save[1], save[2], save[3], save[4]};
    for (const Cand &c : cands) {
        if (smat_fdtd_set_tuning(p, c.fused, c.ty, c.zc, c.ctas, c.ns) != SMAT_OK) continue;
        launch_set(p->d_base, 0, p->stream);
        enqueue_steps(p, 0, 1, false);
        CK(cudaEventRecord(e0, p->stream));
        enqueue_steps(p, 0, nsteps, false);
        CK(cudaEventRecord(e1, p->stream));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (cudaGetLastError() != cudaSuccess) continue; /* a form whose launches were refused */
        if (verbose)
            fprintf(stderr, "autotune: kernel %d tile_y %d z_chunk %d ctas_per_sm %d slots %d: %.4f ms/step\n",
                    c.fused, c.ty, c.zc, c.ctas, c.ns, ms / nsteps);
        if (ms < bms) {
            bms = ms;
            bc = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    p->nq = nq;
    CK(p->cpy(p->d_iI, p->h_iI.data(), sizeof(int) * p->batch, cudaMemcpyHostToDevice));
    CK(cudaStreamSynchronize(p->stream));
    rc = smat_fdtd_set_tuning(p, bc.fused, bc.ty, bc.zc, bc.ctas, bc.ns);
    if (rc) return rc;
    if (best) smat_fdtd_get_tuning(p, best);
    if (best_ms) *best_ms = bms / nsteps;
    return SMAT_OK;
}

extern "C" int smat_device_info(char *name, int name_len, int *sm_count, int *cc)
{
    int dev = 0;
    CK(cudaGetDevice(&dev));
    cudaDeviceProp pr;
    CK(cudaGetDeviceProperties(&pr, dev));
    if (name && name_len > 0) {
        strncpy(name, pr.name, name_len - 1);
        name[name_len - 1] = '\0';
    }
    if (sm_count) *sm_count = pr.multiProcessorCount;
    if (cc) *cc = pr.major * 10 + pr.minor;
    return SMAT_OK;
}

extern "C" int smat_fdtd_get_tuning(const smat_fdtd_plan *p, int out[5])
{
    if (!p || !out) return smat_fail(SMAT_EINVAL, "get_tuning: bad arguments");
    out[0] = p->fused;
    out[1] = p->fused == 6 ? p->ty : p->by32;
    out[2] = p->fused == 6 ? p->zc : p->szc;
    out[3] = p->fused == 6 ? p->ctas_per_sm : p->sweep_mb;
    out[4] = p->ns;
    return SMAT_OK;
}

extern "C" int smat_fdtd_copy_bytes(const smat_fdtd_plan *p, long long *h2d, long long *d2h)
{
    if (!p) return smat_fail(SMAT_EINVAL, "null plan");
    if (h2d) *h2d = p->h2d_bytes;
    if (d2h) *d2h = p->d2h_bytes;
    return SMAT_OK;
}

extern "C" int smat_fdtd_sync(smat_fdtd_plan *p)
{
    if (!p) return smat_fail(SMAT_EINVAL, "null plan");
    CK(cudaStreamSynchronize(p->stream));
    if (p->d_err) {
        int err = 0;
        CK(cudaMemcpy(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
        p->d2h_bytes += sizeof(int);
        if (err) {
            CK(cudaMemset(p->d_err, 0, sizeof(int)));
            return smat_fail(SMAT_ECUDA, err == 2 ? "pipelined sweeps: a wait for an H item timed out"
                                                  : "fused pipeline: a staged plane did not arrive (timed out)");
        }
    }
    return SMAT_OK;
}

static int read_acc(smat_fdtd_plan *p, int b, int f, int q, std::vector<double> &out)
{
    const size_t n = 4 * (size_t)p->pl * 2;
    out.resize(n);
    const double *src = p->d_acc + (((size_t)b * p->nfreq + f) * p->nq + q) * n;
    CK(p->cpy(out.data(), src, n * 8, cudaMemcpyDeviceToHost));
    CK(cudaStreamSynchronize(p->stream));
    return SMAT_OK;
}

extern "C" int smat_fdtd_get_monitor(smat_fdtd_plan *p, int b, double *HB, double *EB, double *HT, double *ET)
{
    smat_clear_error();
    if (!p || b < 0 || b >= p->batch) return smat_fail(SMAT_EINVAL, "get_monitor: bad arguments");
    if (!p->ref_dft) return smat_fail(SMAT_ESTATE, "get_monitor: the reference DFT is not configured");
    std::vector<double> a;
    for (int q = 0; q < 2; q++) {
        int rc = read_acc(p, b, 0, q, a);
        if (rc) return rc;
        double *Hd = q ? HT : HB, *Ed = q ? ET : EB;
        for (long long px = 0; px < p->pl; px++)
            for (int v = 0; v < 2; v++) {
                if (Hd) {
                    Hd[2 * (v + 2 * px)] = a[2 * (v * p->pl + px)];
                    Hd[2 * (v + 2 * px) + 1] = a[2 * (v * p->pl + px) + 1];
                }
                if (Ed) {
                    Ed[2 * (v + 2 * px)] = a[2 * ((2 + v) * p->pl + px)];
                    Ed[2 * (v + 2 * px) + 1] = a[2 * ((2 + v) * p->pl + px) + 1];
                }
            }
    }
    return SMAT_OK;
}

/* preload the reference DFT accumulators (used by smat_main_calc, whose
 * caller's HB..ET carry the running sums) */
static int set_monitor(smat_fdtd_plan *p, const double *HB, const double *EB, const double *HT, const double *ET)
{
    const size_t n = 4 * (size_t)p->pl * 2;
    std::vector<double> a(n);
    for (int q = 0; q < 2; q++) {
        const double *Hs = q ? HT : HB, *Es = q ? ET : EB;
        for (long long px = 0; px < p->pl; px++)
            for (int v = 0; v < 2; v++) {
                a[2 * (v * p->pl + px)] = Hs[2 * (v + 2 * px)];
                a[2 * (v * p->pl + px) + 1] = Hs[2 * (v + 2 * px) + 1];
                a[2 * ((2 + v) * p->pl + px)] = Es[2 * (v + 2 * px)];
                a[2 * ((2 + v) * p->pl + px) + 1] = Es[2 * (v + 2 * px) + 1];
            }
        CK(p->cpy(p->d_acc + q * n, a.data(), n * 8, cudaMemcpyHostToDevice));
        CK(cudaStreamSynchronize(p->stream));
    }
    return SMAT_OK;
}

extern "C" int smat_fdtd_get_dft(smat_fdtd_plan *p, int b, int f, int q, double *out)
{
    smat_clear_error();
    if (!p || !out || b < 0 || b >= p->batch || f < 0 || f >= p->nfreq || q < 0 || q >= p->nq)
        return smat_fail(SMAT_EINVAL, "get_dft: bad arguments");
    std::vector<double> a;
    int rc = read_acc(p, b, f, q, a);
    if (rc) return rc;
    memcpy(out, a.data(), a.size() * 8);
    return SMAT_OK;
}

extern "C" int smat_fdtd_dft_count(const smat_fdtd_plan *p, int *nfreq, int *nplanes)
{
    if (!p) return smat_fail(SMAT_EINVAL, "null plan");
    if (nfreq) *nfreq = p->nfreq;
    if (nplanes) *nplanes = p->nq;
    return SMAT_OK;
}

extern "C" int smat_fdtd_dft_device(smat_fdtd_plan *p, int b, int f, int q, const double **ptr, long long *fstride)
{
    if (!p || !ptr || b < 0 || b >= p->batch || f < 0 || f >= p->nfreq || q < 0 || q >= p->nq)
        return smat_fail(SMAT_EINVAL, "dft_device: bad arguments");
    *ptr = p->d_acc + 2 * ((((size_t)b * p->nfreq + f) * p->nq + q) * 4 * (size_t)p->pl);
    if (fstride) *fstride = (long long)p->nq * 4 * p->pl;
    return SMAT_OK;
}

extern "C" int smat_fdtd_check_finite(smat_fdtd_plan *p, int *finite, double *max_abs)
{
    smat_clear_error();
    if (!p) return smat_fail(SMAT_EINVAL, "null plan");
    CK(cudaMemsetAsync(p->d_scratch, 0, 8, p->stream));
    const bool d = p->precision == SMAT_FP64;
    const long long nf = (long long)p->batch * 3 * p->n3;
    const long long na = d ? (long long)p->batch * 3 * (p->lnotn + 1) : nf;
    const P32 q = make_p32(p, false);
    const void *arr[4] = {d ? (void *)p->d_H64 : (void *)q.H, d ? (void *)p->d_E64 : (void *)q.E,
                          d ? (void *)p->d_Ha64 : (void *)q.Ha, d ? (void *)p->d_Ea64 : (void *)q.Ea};
    for (int i = 0; i < 4; i++) launch_maxabs(arr[i], i < 2 ? nf : na, d, p->d_scratch, p->stream);
    unsigned long long bits = 0;
    CK(p->cpy(&bits, p->d_scratch, 8, cudaMemcpyDeviceToHost));
    CK(cudaStreamSynchronize(p->stream));
    double m;
    memcpy(&m, &bits, 8);
    if (finite) *finite = std::isfinite(m) ? 1 : 0;
    if (max_abs) *max_abs = m;
    return SMAT_OK;
}

extern "C" int smat_main_calc(const int L[4], const double *Ah, const double *Bh, const double *Ae, const double *Be,
                              const int iBc[3], double *H_t, double *E_t, const int iBTIin[4], const double *Hi,
                              const double *Ei, const double *ExpN2, double *HB, double *EB, double *HT, double *ET,
                              const char *Cont, const int *address_notn)
{
    smat_clear_error();
    if (!L || !H_t || !E_t || !Hi || !Ei || !ExpN2 || !HB || !EB || !HT || !ET || !Cont || !address_notn)
        return smat_fail(SMAT_EINVAL, "main_calc: null argument");
    const long long n3 = (long long)L[0] * L[1] * L[2];
    int lnotn = 0;
    for (long long l = 0; l < n3; l++) lnotn += Cont[l] != 'n';
    smat_fdtd_plan *p = nullptr;
    int rc = smat_fdtd_create_from_coeffs(L, Ah, Bh, Ae, Be, iBc, Cont, address_notn, lnotn, iBTIin, 1, nullptr, &p);
    if (rc) return rc;
    rc = smat_fdtd_set_fields(p, 0, H_t, E_t);
    if (!rc) rc = set_monitor(p, HB, EB, HT, ET);
    if (!rc) rc = smat_fdtd_step(p, Hi, Ei, ExpN2);
    if (!rc) rc = smat_fdtd_get_fields(p, 0, H_t, E_t);
    if (!rc) rc = smat_fdtd_get_monitor(p, 0, HB, EB, HT, ET);
    smat_fdtd_destroy(p);
    return rc;
}

/* ---- checkpoint and resume ------------------------------------------------ */

namespace {

struct StateHeader {
    char magic[8];
    int32_t version, precision, batch, L[4], lnotn, nfreq, nq;
    int32_t cur; /* FP32: the field set that holds the state */
    int32_t reserved[4];
};

constexpr char STATE_MAGIC[8] = {'S', 'M', 'A', 'T', 'S', 'T', 'A', 'T'};

/* the device arrays that hold a plan's state, in file order */
std::vector<std::pair<void *, size_t>> state_arrays(smat_fdtd_plan *p)
{
    std::vector<std::pair<void *, size_t>> a;
    const size_t b = (size_t)p->batch, n3 = (size_t)p->n3;
    if (p->precision == SMAT_FP64) {
        const size_t main = b * 3 * n3 * 8, aux = b * 3 * ((size_t)p->lnotn + 1) * 8;
        a.push_back({p->d_H64, main});
        a.push_back({p->d_E64, main});
        a.push_back({p->d_Ha64, aux});
        a.push_back({p->d_Ea64, aux});
    } else {
        const P32 q = make_p32(p, false);
        const size_t f = b * 3 * n3 * 4;
        a.push_back({q.H, f});
        a.push_back({q.E, f});
        a.push_back({q.Ha, f});
        a.push_back({q.Ea, f});
    }
    if (p->d_acc && p->nq > 0 && p->nfreq > 0)
        a.push_back({p->d_acc, b * (size_t)p->nfreq * p->nq * 4 * (size_t)p->pl * 16});
    return a;
}

void fill_header(const smat_fdtd_plan *p, StateHeader &h)
{
    memset(&h, 0, sizeof h);
    memcpy(h.magic, STATE_MAGIC, 8);
    h.version = 1;
    h.precision = p->precision;
    h.batch = p->batch;
    for (int i = 0; i < 4; i++) h.L[i] = p->L[i];
    h.lnotn = p->lnotn;
    h.nfreq = p->d_acc ? p->nfreq : 0;
    h.nq = p->d_acc ? p->nq : 0;
    h.cur = p->precision == SMAT_FP32 ? p->cur : 0;
}

} // namespace

extern "C" int smat_fdtd_save_state(smat_fdtd_plan *p, const char *path)
{
    smat_clear_error();
    if (!p || !path) return smat_fail(SMAT_EINVAL, "save_state: bad arguments");
    CK(cudaStreamSynchronize(p->stream));
    StateHeader h;
    fill_header(p, h);
    FILE *f = fopen(path, "wb");
    if (!f) return smat_fail(SMAT_EINVAL, "save_state: cannot open %s", path);
    int rc = fwrite(&h, sizeof h, 1, f) == 1 ? SMAT_OK : smat_fail(SMAT_EINVAL, "save_state: write error");
    std::vector<char> buf;
    for (const auto &a : state_arrays(p)) {
        if (rc) break;
        buf.resize(a.second);
        p->d2h_bytes += (long long)a.second;
        if (cudaMemcpy(buf.data(), a.first, a.second, cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "save_state: copy");
            break;
        }
        if (fwrite(buf.data(), 1, a.second, f) != a.second) rc = smat_fail(SMAT_EINVAL, "save_state: write error");
    }
    if (fclose(f) != 0 && !rc) rc = smat_fail(SMAT_EINVAL, "save_state: write error");
    return rc;
}

extern "C" int smat_fdtd_load_state(smat_fdtd_plan *p, const char *path)
{
    smat_clear_error();
    if (!p || !path) return smat_fail(SMAT_EINVAL, "load_state: bad arguments");
    CK(cudaStreamSynchronize(p->stream));
    FILE *f = fopen(path, "rb");
    if (!f) return smat_fail(SMAT_EINVAL, "load_state: cannot open %s", path);
    StateHeader h, want;
    fill_header(p, want);
    int rc = SMAT_OK;
    if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, STATE_MAGIC, 8) != 0 || h.version != 1)
        rc = smat_fail(SMAT_EINVAL, "load_state: %s is not a state file", path);
    else if (h.precision != want.precision || h.batch != want.batch || memcmp(h.L, want.L, sizeof h.L) != 0 ||
             h.lnotn != want.lnotn || h.nfreq != want.nfreq || h.nq != want.nq)
        rc = smat_fail(SMAT_EINVAL, "load_state: %s holds another plan's state (grid, precision, batch, split "
                                    "cells or DFT setup differ)", path);
    else if (h.cur != 0 && h.cur != 1)
        rc = smat_fail(SMAT_EINVAL, "load_state: %s is not a state file", path);
    /* FP32: into the field set it was saved from, so that a run continues with
     * the same set parity (and so the same grouping of the DFT ring's sums) */
    if (!rc && p->precision == SMAT_FP32) p->cur = h.cur;
    std::vector<char> buf;
    for (const auto &a : state_arrays(p)) {
        if (rc) break;
        buf.resize(a.second);
        if (fread(buf.data(), 1, a.second, f) != a.second) {
            rc = smat_fail(SMAT_EINVAL, "load_state: %s is truncated", path);
            break;
        }
        p->h2d_bytes += (long long)a.second;
        if (cudaMemcpy(a.first, buf.data(), a.second, cudaMemcpyHostToDevice) != cudaSuccess)
            rc = cuda_fail(cudaGetLastError(), "load_state: copy");
    }
    if (!rc && fgetc(f) != EOF) rc = smat_fail(SMAT_EINVAL, "load_state: %s has trailing data", path);
    fclose(f);
    if (!rc) drop_graph(p);
    return rc;
}
