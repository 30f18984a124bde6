/*
 * FP32 split-field FDTD step (bandwidth path) in total-field form.
 *
 * Same update as the reference main_calc (FDTDcalc/FDTDsplitfieldMetal.c:
 * 242-329), rewritten so that the hot loop reads one array per component:
 *
 *   T = main + aux.  Every curl in the reference of an ordinary or split cell
 *   is curl(main) + curl(aux) over the same stencil (ope_R + ope_Rmap), i.e.
 *   curl(T).  So neighbours read T only; the aux slot is touched only by the
 *   cell that owns it.
 *
 *   ordinary cell ('n'), lossless:  F <- F -/+ B * curl(T)   (A == 1 exactly)
 *   split cell ('a'):   p = T - aux, m = aux
 *                       p <- A(s_{c+1}) p -/+ B G(s_{c+1}) curl_{+}(T)
 *                       m <- A(s_{c+2}) m -/+ B G(s_{c+2}) curl_{-}(T)
 *                       T <- p + m, aux <- m
 *     with A(s) = (tR - tI s)/(tR + tI s), G(s) = tR/(tR + tI s), the exact
 *     factorisation of the reference coefficients (:118-127) for real media;
 *     B = 1/(tR Re mu) per cell and component, A and G from 1-D sigma tables.
 *   anything else (lossy or PEC ordinary cells, lossy split cells, the stable
 *   form of 'h'/'e'/'b' cells and their frozen components) runs from a
 *   per-cell record; such cells are marked by NaN in their first coefficient.
 *
 * Monitor-plane samples go to a ring of K steps; a flush kernel folds the ring
 * into the FP64 DFT accumulators (FP32 partial sums over K terms).
 */
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"

namespace smat {

__device__ __forceinline__ double sheet32(const Src &s, int pl, int b, int k, bool efield, int v, int p)
{
    if (s.xsrc) return s.xsrc[(efield ? 2 * pl : 0) + v + 2 * p];
    const double *sc = s.sched + 6 * (long long)k + (efield ? 0 : 3);
    const double *w = s.inc + (long long)b * 8 * pl + (efield ? 4 * pl : 0) + 2 * (v + 2 * p);
    return sc[0] * (sc[1] * w[0] + sc[2] * w[1]);
}

__device__ __forceinline__ int monitor_index(const Dft &d, int j2)
{
    int q = -1;
#pragma unroll
    for (int i = 0; i < MAX_PLANES; i++)
        if (i < d.nq && d.planes[i] == j2) q = i;
    return q;
}

__device__ __forceinline__ float *ring_at(const Dft &d, int pl, int b, int k, int q, int v)
{
    const int slot = k % d.ringK;
    return d.ring + ((((long long)b * d.ringK + slot) * d.nq + q) * 4 + v) * (long long)pl;
}

/* One sweep.  EF = false: H from E (backward curls, sign -); EF = true: E from
 * H (forward curls, sign +; the stable form uses backward curls, :310). */
template <bool EF>
__global__ void __launch_bounds__(256) k_sweep32(const P32 p, const int rel, const int z0)
{
    /* blockIdx.y = row block * batch + excitation: the blocks of one tile for
     * all excitations launch together and share the coefficient lines in L2 */
    const int b = blockIdx.y % p.batch;
    const int j0 = blockIdx.x * 32 + threadIdx.x, j1 = (blockIdx.y / p.batch) * blockDim.y + threadIdx.y;
    const int j2 = z0 + blockIdx.z;
    const Geo &g = p.g;
    if (j0 >= g.L0 || j1 >= g.L1) return;
    const long long n3 = g.n3, l = j0 + (long long)g.L0 * (j1 + (long long)g.L1 * j2);
    const float *__restrict__ cf = EF ? p.be : p.bh;
    float *__restrict__ F0 = EF ? p.E : p.H;   /* updated field (total form) */
    float *__restrict__ Fa0 = EF ? p.Ea : p.Ha;
    const float *__restrict__ G0 = EF ? p.H : p.E; /* field whose curl drives it */
    const float *__restrict__ Ga0 = EF ? p.Ha : p.Ea;
    const float sg = EF ? 1.0f : -1.0f;
    const int k = *p.s.base + rel;
    const int q = monitor_index(p.d, j2);
    const int px = j0 + g.L0 * j1;
    const long long bs = 3 * n3;
    /* issue every load of the common paths before any branch, so a thread
     * waits for DRAM once: its coefficients, its own field, the six curl
     * neighbours and the PML masks */
    const float c0 = cf[l], c1 = cf[n3 + l], c2 = cf[2 * n3 + l];
    const int S = g.L0 + g.L1 + g.L2, s1 = g.L0, s2 = g.L0 + g.L1;
    const bool split = p.pmask[j0] | p.pmask[s1 + j1] | p.pmask[s2 + j2];
    const Stn32 st = make_stn32(g, j0, j1, j2, EF);
    float *F = F0 + b * bs, *Fa = Fa0 + b * bs;
    const float *G = G0 + b * bs;
    float pl[3], mi[3], fo[3];
    {
        auto get = [&](int c, long long o) { return G[c * n3 + l + o]; };
        curl32<EF>(get, st, pl, mi);
#pragma unroll
        for (int c = 0; c < 3; c++) fo[c] = F[c * n3 + l];
    }

    if (!isnan(c0)) {
        const float bn[3] = {c0, c1, c2};
        if (!split) {
            float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
            if (j2 == p.s.iI[b]) {
                W[0] += (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 1, px));
                W[1] -= (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 0, px));
            }
            float f[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                f[c] = fmaf(sg * bn[c], W[c], fo[c]);
                F[c * n3 + l] = f[c];
            }
            if (q >= 0) {
                ring_at(p.d, g.pl, b, k, q, EF ? 2 : 0)[px] = f[0];
                ring_at(p.d, g.pl, b, k, q, EF ? 3 : 1)[px] = f[1];
            }
        } else {
            const int jx[3] = {j0, s1 + j1, s2 + j2};
            const float *tA = p.tab + (EF ? 2 : 0) * S, *tG = p.tab + (EF ? 3 : 1) * S;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int i1 = jx[(c + 1) % 3], i2 = jx[(c + 2) % 3];
                const float Ap = tA[i1], Bp = sg * bn[c] * tG[i1];
                const float Am = tA[i2], Bm = sg * bn[c] * tG[i2];
                const float m = Fa[c * n3 + l];
                const float pp = fo[c] - m;
                const float np = fmaf(Bp, pl[c], Ap * pp);
                const float nm = fmaf(Bm, mi[c], Am * m);
                F[c * n3 + l] = np + nm;
                Fa[c * n3 + l] = nm;
                if (q >= 0 && c < 2) ring_at(p.d, g.pl, b, k, q, (EF ? 2 : 0) + c)[px] = np + nm;
            }
        }
        return;
    }

    /* general cells */
    const Rec32 r = (EF ? p.erec : p.hrec)[__float_as_int(c1)];
    const bool stable = r.kind == RK_STABLE;
    {
        const Stn32 sts = make_stn32(g, j0, j1, j2, EF && !stable);
        const float *Ga = Ga0 + b * bs;
        float main_out[3];
        if (r.kind == RK_FROZEN) {
#pragma unroll
            for (int c = 0; c < 3; c++) main_out[c] = F[c * n3 + l] - Fa[c * n3 + l];
        } else if (stable) {
            /* the stable form differentiates the MAIN slot of the other field */
            auto get = [&](int c, long long o) { return G[c * n3 + l + o] - Ga[c * n3 + l + o]; };
            curl32<false>(get, sts, pl, mi);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const float W = pl[c] + mi[c];
                float x = Fa[c * n3 + l];
                float f = F[c * n3 + l] - x;
                f += 0.5f * x;
                x = fmaf(sg * r.B1[c], W, r.A1[c] * x);
                f += 0.5f * x;
                main_out[c] = f;
                F[c * n3 + l] = f + x;
                Fa[c * n3 + l] = x;
            }
        } else {
            if (r.kind == RK_N) {
                float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
                if (j2 == p.s.iI[b]) {
                    W[0] += (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 1, px));
                    W[1] -= (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 0, px));
                }
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float f = fmaf(sg * r.B0[c], W[c], r.A0[c] * F[c * n3 + l]);
                    F[c * n3 + l] = f;
                    main_out[c] = f;
                }
            } else { /* RK_A: split cell with lossy media */
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float m = Fa[c * n3 + l];
                    const float pp = F[c * n3 + l] - m;
                    const float np = fmaf(sg * r.B0[c], pl[c], r.A0[c] * pp);
                    const float nm = fmaf(sg * r.B1[c], mi[c], r.A1[c] * m);
                    F[c * n3 + l] = np + nm;
                    Fa[c * n3 + l] = nm;
                    main_out[c] = np + nm; /* a plane through the PML samples the total field */
                }
            }
        }
        if (q >= 0) {
            ring_at(p.d, g.pl, b, k, q, EF ? 2 : 0)[px] = main_out[0];
            ring_at(p.d, g.pl, b, k, q, EF ? 3 : 1)[px] = main_out[1];
        }
    }
}

/* ---------------------------------------------------------------------------
 * Vectorised sweep: four consecutive x-cells per thread (float4 loads and
 * stores), for L0 % 4 == 0.  Every element is updated with exactly the
 * expressions of k_sweep32, so the two kernels give the same bits; what changes
 * is that a thread keeps four cells' worth of loads in flight, which is what
 * the HBM needs (the six curl neighbours of a cell are mostly cache hits, so a
 * one-cell thread has only ~25 B of DRAM reads outstanding).  The x
 * neighbours come from the adjacent lane by warp shuffle.
 * ------------------------------------------------------------------------- */
__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float el(const float4 &v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }
__device__ __forceinline__ void set_el(float4 &v, int i, float x)
{
    if (i == 0) v.x = x;
    else if (i == 1) v.y = x;
    else if (i == 2) v.z = x;
    else v.w = x;
}
__device__ __forceinline__ float4 scale4(float4 v, float f) { return make_float4(f * v.x, f * v.y, f * v.z, f * v.w); }

/* loads of the other field: CG = true reads through L2 only (ld.global.cg),
 * for data another CTA of the same launch may have written */
template <bool CG> __device__ __forceinline__ float4 ldG4(const float *p)
{
    return CG ? __ldcg(reinterpret_cast<const float4 *>(p)) : *reinterpret_cast<const float4 *>(p);
}
template <bool CG> __device__ __forceinline__ float ldG(const float *p) { return CG ? __ldcg(p) : *p; }

/* The loads of one quad row segment (cells x = xr..xr+3 of row j1, plane j2,
 * excitation b; a warp covers 128 consecutive x-cells, lane = threadIdx.x % 32)
 * into q, including the x neighbours by warp shuffle.  False for a row past
 * the grid (uniform per warp). */
struct QIn {
    float4 c[3], out[3], gh[3], aux[3], gy0, gy2, gz0, gz1;
    float xn1, xn2;
    long long l;
    int x0;
    bool live, qsplit, pyz;
};

template <bool EF, bool CG>
__device__ __forceinline__ bool quad_load(const P32 &p, const int b, const int j1, const int j2, const int xr, QIn &q)
{
    const Geo &g = p.g;
    if (j1 >= g.L1) return false; /* uniform per warp */
    const bool live = xr < g.L0;
    const int x0 = live ? xr : g.L0 - 4; /* idle lanes load valid data, store nothing */
    const long long n3 = g.n3, bs = 3 * n3;
    const long long l = x0 + (long long)g.L0 * (j1 + (long long)g.L1 * j2);
    const float *__restrict__ cf = EF ? p.be : p.bh;
    const float *__restrict__ F = (EF ? p.E : p.H) + b * bs;
    const float *__restrict__ Fa = (EF ? p.Ea : p.Ha) + b * bs;
    const float *__restrict__ G = (EF ? p.H : p.E) + b * bs;
    const int s1 = g.L0, s2 = g.L0 + g.L1;
    /* neighbours along y and z (whole quads) with the boundary factor */
    const bool ey = EF ? (j1 + 1 == g.L1) : (j1 == 0);
    const bool ez = EF ? (j2 + 1 == g.L2) : (j2 == 0);
    const long long oy = (long long)g.L0 * (EF ? (ey ? -(g.L1 - 1) : 1) : (ey ? g.L1 - 1 : -1));
    const long long oz = (long long)g.pl * (EF ? (ez ? -(g.L2 - 1) : 1) : (ez ? g.L2 - 1 : -1));
    const float fy = ey ? (float)g.bc[1] : 1.0f, fz = ez ? (float)g.bc[2] : 1.0f;

    /* split-PML quads need their aux slots: decided from the 1-D masks before
     * any load, so that those loads leave with the others (one DRAM round trip) */
    const bool pyz = p.pmask[s1 + j1] | p.pmask[s2 + j2];
    const bool qsplit = pyz | p.pmask[x0] | p.pmask[x0 + 1] | p.pmask[x0 + 2] | p.pmask[x0 + 3];
    q.pyz = pyz;
    q.qsplit = qsplit;
    q.live = live;
    q.x0 = x0;
    q.l = l;
    float4 *c = q.c, *out = q.out, *gh = q.gh, *aux = q.aux;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        c[i] = ld4(cf + i * n3 + l);
        out[i] = ld4(F + i * n3 + l);
        gh[i] = ldG4<CG>(G + i * n3 + l);
    }
    if (qsplit) {
#pragma unroll
        for (int i = 0; i < 3; i++) aux[i] = ld4(Fa + i * n3 + l);
    }
    /* H sweep: Ex, Ez at y-1; Ex, Ey at z-1.  E sweep: Hx, Hz at y+1; Hx, Hy at z+1. */
    q.gy0 = scale4(ldG4<CG>(G + 0 * n3 + l + oy), fy);
    q.gy2 = scale4(ldG4<CG>(G + 2 * n3 + l + oy), fy);
    q.gz0 = scale4(ldG4<CG>(G + 0 * n3 + l + oz), fz);
    q.gz1 = scale4(ldG4<CG>(G + 1 * n3 + l + oz), fz);
    /* x neighbours: H sweep needs Ey, Ez at x-1; E sweep Hy, Hz at x+1 */
    const unsigned full = 0xffffffffu;
    float &xn1 = q.xn1, &xn2 = q.xn2; /* component 1, 2 of the outer neighbour of the quad */
    if (!EF) {
        xn1 = __shfl_up_sync(full, gh[1].w, 1);
        xn2 = __shfl_up_sync(full, gh[2].w, 1);
        if ((threadIdx.x & 31) == 0 || x0 == 0) {
            const bool edge = x0 == 0;
            const long long o = edge ? g.L0 - 1 : -1;
            const float f = edge ? (float)g.bc[0] : 1.0f;
            xn1 = f * ldG<CG>(G + 1 * n3 + l + o);
            xn2 = f * ldG<CG>(G + 2 * n3 + l + o);
        }
    } else {
        xn1 = __shfl_down_sync(full, gh[1].x, 1);
        xn2 = __shfl_down_sync(full, gh[2].x, 1);
        if ((threadIdx.x & 31) == 31 || x0 + 4 == g.L0) {
            const bool edge = x0 + 4 == g.L0;
            const long long o = edge ? -(g.L0 - 4) : 4;
            const float f = edge ? (float)g.bc[0] : 1.0f;
            xn1 = f * ldG<CG>(G + 1 * n3 + l + o);
            xn2 = f * ldG<CG>(G + 2 * n3 + l + o);
        }
    }
    return true;
}

/* The update and stores of a quad loaded by quad_load (same expressions as
 * k_sweep32: the same bits) */
template <bool EF>
__device__ __forceinline__ void quad_compute(const P32 &p, const int rel, const int b, const int j1, const int j2,
                                             QIn &qi)
{
    if (!qi.live) return;
    const Geo &g = p.g;
    const long long n3 = g.n3, bs = 3 * n3, l = qi.l;
    const int x0 = qi.x0;
    float *__restrict__ F = (EF ? p.E : p.H) + b * bs;
    float *__restrict__ Fa = (EF ? p.Ea : p.Ha) + b * bs;
    const float sg = EF ? 1.0f : -1.0f;
    const int k = *p.s.base + rel;
    const int px0 = x0 + g.L0 * j1;
    const int S = g.L0 + g.L1 + g.L2, s1 = g.L0, s2 = g.L0 + g.L1;
    const bool pyz = qi.pyz, qsplit = qi.qsplit;
    float4 *c = qi.c, *out = qi.out, *gh = qi.gh, *aux = qi.aux;
    const float4 gy0 = qi.gy0, gy2 = qi.gy2, gz0 = qi.gz0, gz1 = qi.gz1;
    const float xn1 = qi.xn1, xn2 = qi.xn2;
    const bool on_src = j2 == p.s.iI[b];
    const int q = monitor_index(p.d, j2);
    bool any_aux = false;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int xx = x0 + i;
        const float h0 = el(gh[0], i), h1 = el(gh[1], i), h2 = el(gh[2], i);
        /* neighbour along x of element i */
        float n1x, n2x;
        if (!EF) {
            n1x = i == 0 ? xn1 : el(gh[1], i - 1);
            n2x = i == 0 ? xn2 : el(gh[2], i - 1);
        } else {
            n1x = i == 3 ? xn1 : el(gh[1], i + 1);
            n2x = i == 3 ? xn2 : el(gh[2], i + 1);
        }
        float pl[3], mi[3];
        if (!EF) { /* backward, as curl32<false> */
            pl[0] = h2 - el(gy2, i);
            mi[0] = el(gz1, i) - h1;
            pl[1] = h0 - el(gz0, i);
            mi[1] = n2x - h2;
            pl[2] = h1 - n1x;
            mi[2] = el(gy0, i) - h0;
        } else { /* forward, as curl32<true> */
            pl[0] = el(gy2, i) - h2;
            mi[0] = h1 - el(gz1, i);
            pl[1] = el(gz0, i) - h0;
            mi[1] = h2 - n2x;
            pl[2] = n1x - h1;
            mi[2] = h0 - el(gy0, i);
        }
        const float c0 = el(c[0], i);
        if (isnan(c0)) { /* general cell: rewritten by k_general32 after this launch */
            any_aux = true;
            continue;
        }
        const bool split = p.pmask[xx] | pyz;
        const float bn[3] = {c0, el(c[1], i), el(c[2], i)};
        if (!split) {
            float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
            if (on_src) {
                W[0] += (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 1, px0 + i));
                W[1] -= (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 0, px0 + i));
            }
#pragma unroll
            for (int cc = 0; cc < 3; cc++) set_el(out[cc], i, fmaf(sg * bn[cc], W[cc], el(out[cc], i)));
        } else {
            any_aux = true;
        }
    }
    /* elements that need their aux slot (split) or a record (general) */
    if (any_aux) {
        if (!qsplit) { /* a general (record) cell in an unsplit quad: rare */
#pragma unroll
            for (int cc = 0; cc < 3; cc++) aux[cc] = ld4(Fa + cc * n3 + l);
        }
        const int jy = s1 + j1, jz = s2 + j2;
        const float *tA = p.tab + (EF ? 2 : 0) * S, *tG = p.tab + (EF ? 3 : 1) * S;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int xx = x0 + i;
            const float c0 = el(c[0], i);
            if (isnan(c0)) continue;
            if (!(p.pmask[xx] | pyz)) continue;
            const float h0 = el(gh[0], i), h1 = el(gh[1], i), h2 = el(gh[2], i);
            float n1x, n2x;
            if (!EF) {
                n1x = i == 0 ? xn1 : el(gh[1], i - 1);
                n2x = i == 0 ? xn2 : el(gh[2], i - 1);
            } else {
                n1x = i == 3 ? xn1 : el(gh[1], i + 1);
                n2x = i == 3 ? xn2 : el(gh[2], i + 1);
            }
            float pl[3], mi[3];
            if (!EF) {
                pl[0] = h2 - el(gy2, i);
                mi[0] = el(gz1, i) - h1;
                pl[1] = h0 - el(gz0, i);
                mi[1] = n2x - h2;
                pl[2] = h1 - n1x;
                mi[2] = el(gy0, i) - h0;
            } else {
                pl[0] = el(gy2, i) - h2;
                mi[0] = h1 - el(gz1, i);
                pl[1] = el(gz0, i) - h0;
                mi[1] = h2 - n2x;
                pl[2] = n1x - h1;
                mi[2] = h0 - el(gy0, i);
            }
            const int jx[3] = {xx, jy, jz};
            const float bn[3] = {c0, el(c[1], i), el(c[2], i)};
#pragma unroll
            for (int cc = 0; cc < 3; cc++) {
                const int i1 = jx[(cc + 1) % 3], i2 = jx[(cc + 2) % 3];
                const float Ap = tA[i1], Bp = sg * bn[cc] * tG[i1];
                const float Am = tA[i2], Bm = sg * bn[cc] * tG[i2];
                const float m = el(aux[cc], i);
                const float pp = el(out[cc], i) - m; /* out still holds the old field here */
                const float np = fmaf(Bp, pl[cc], Ap * pp);
                const float nm = fmaf(Bm, mi[cc], Am * m);
                set_el(out[cc], i, np + nm);
                set_el(aux[cc], i, nm);
            }
        }
    }
#pragma unroll
    for (int cc = 0; cc < 3; cc++) st4(F + cc * n3 + l, out[cc]);
    if (any_aux) {
#pragma unroll
        for (int cc = 0; cc < 3; cc++) st4(Fa + cc * n3 + l, aux[cc]);
    }
    if (q >= 0) {
        /* split elements sample the total field, ordinary ones their field */
        st4(ring_at(p.d, g.pl, b, k, q, EF ? 2 : 0) + px0, out[0]);
        st4(ring_at(p.d, g.pl, b, k, q, EF ? 3 : 1) + px0, out[1]);
    }
}

/* one quad row segment: cells x = xr..xr+3 of row j1, plane j2, excitation b;
 * a warp covers 128 consecutive x-cells (lane = threadIdx.x) */
template <bool EF, bool CG>
__device__ __forceinline__ void sweep32v_quad(const P32 &p, const int rel, const int b, const int j1, const int j2,
                                              const int xr)
{
    const Geo &g = p.g;
    if (j1 >= g.L1) return; /* uniform per warp */
    const bool live = xr < g.L0;
    const int x0 = live ? xr : g.L0 - 4; /* idle lanes load valid data, store nothing */
    const long long n3 = g.n3, bs = 3 * n3;
    const long long l = x0 + (long long)g.L0 * (j1 + (long long)g.L1 * j2);
    const float *__restrict__ cf = EF ? p.be : p.bh;
    float *__restrict__ F = (EF ? p.E : p.H) + b * bs;
    float *__restrict__ Fa = (EF ? p.Ea : p.Ha) + b * bs;
    const float *__restrict__ G = (EF ? p.H : p.E) + b * bs;
    const float sg = EF ? 1.0f : -1.0f;
    const int k = *p.s.base + rel;
    const int px0 = x0 + g.L0 * j1;
    const int S = g.L0 + g.L1 + g.L2, s1 = g.L0, s2 = g.L0 + g.L1;
    /* neighbours along y and z (whole quads) with the boundary factor */
    const bool ey = EF ? (j1 + 1 == g.L1) : (j1 == 0);
    const bool ez = EF ? (j2 + 1 == g.L2) : (j2 == 0);
    const long long oy = (long long)g.L0 * (EF ? (ey ? -(g.L1 - 1) : 1) : (ey ? g.L1 - 1 : -1));
    const long long oz = (long long)g.pl * (EF ? (ez ? -(g.L2 - 1) : 1) : (ez ? g.L2 - 1 : -1));
    const float fy = ey ? (float)g.bc[1] : 1.0f, fz = ez ? (float)g.bc[2] : 1.0f;

    /* split-PML quads need their aux slots: decided from the 1-D masks before
     * any load, so that those loads leave with the others (one DRAM round trip) */
    const bool pyz = p.pmask[s1 + j1] | p.pmask[s2 + j2];
    const bool qsplit = pyz | p.pmask[x0] | p.pmask[x0 + 1] | p.pmask[x0 + 2] | p.pmask[x0 + 3];
    float4 c[3], out[3], gh[3], aux[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        c[i] = ld4(cf + i * n3 + l);
        out[i] = ld4(F + i * n3 + l);
        gh[i] = ldG4<CG>(G + i * n3 + l);
    }
    if (qsplit) {
#pragma unroll
        for (int i = 0; i < 3; i++) aux[i] = ld4(Fa + i * n3 + l);
    }
    /* H sweep: Ex, Ez at y-1; Ex, Ey at z-1.  E sweep: Hx, Hz at y+1; Hx, Hy at z+1. */
    const float4 gy0 = scale4(ldG4<CG>(G + 0 * n3 + l + oy), fy), gy2 = scale4(ldG4<CG>(G + 2 * n3 + l + oy), fy);
    const float4 gz0 = scale4(ldG4<CG>(G + 0 * n3 + l + oz), fz), gz1 = scale4(ldG4<CG>(G + 1 * n3 + l + oz), fz);
    /* x neighbours: H sweep needs Ey, Ez at x-1; E sweep Hy, Hz at x+1 */
    const unsigned full = 0xffffffffu;
    float xn1, xn2; /* component 1, 2 of the outer neighbour of the quad */
    if (!EF) {
        xn1 = __shfl_up_sync(full, gh[1].w, 1);
        xn2 = __shfl_up_sync(full, gh[2].w, 1);
        if ((threadIdx.x & 31) == 0 || x0 == 0) {
            const bool edge = x0 == 0;
            const long long o = edge ? g.L0 - 1 : -1;
            const float f = edge ? (float)g.bc[0] : 1.0f;
            xn1 = f * ldG<CG>(G + 1 * n3 + l + o);
            xn2 = f * ldG<CG>(G + 2 * n3 + l + o);
        }
    } else {
        xn1 = __shfl_down_sync(full, gh[1].x, 1);
        xn2 = __shfl_down_sync(full, gh[2].x, 1);
        if ((threadIdx.x & 31) == 31 || x0 + 4 == g.L0) {
            const bool edge = x0 + 4 == g.L0;
            const long long o = edge ? -(g.L0 - 4) : 4;
            const float f = edge ? (float)g.bc[0] : 1.0f;
            xn1 = f * ldG<CG>(G + 1 * n3 + l + o);
            xn2 = f * ldG<CG>(G + 2 * n3 + l + o);
        }
    }
    if (!live) return;
    const bool on_src = j2 == p.s.iI[b];
    const int q = monitor_index(p.d, j2);
    bool any_aux = false;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int xx = x0 + i;
        const float h0 = el(gh[0], i), h1 = el(gh[1], i), h2 = el(gh[2], i);
        /* neighbour along x of element i */
        float n1x, n2x;
        if (!EF) {
            n1x = i == 0 ? xn1 : el(gh[1], i - 1);
            n2x = i == 0 ? xn2 : el(gh[2], i - 1);
        } else {
            n1x = i == 3 ? xn1 : el(gh[1], i + 1);
            n2x = i == 3 ? xn2 : el(gh[2], i + 1);
        }
        float pl[3], mi[3];
        if (!EF) { /* backward, as curl32<false> */
            pl[0] = h2 - el(gy2, i);
            mi[0] = el(gz1, i) - h1;
            pl[1] = h0 - el(gz0, i);
            mi[1] = n2x - h2;
            pl[2] = h1 - n1x;
            mi[2] = el(gy0, i) - h0;
        } else { /* forward, as curl32<true> */
            pl[0] = el(gy2, i) - h2;
            mi[0] = h1 - el(gz1, i);
            pl[1] = el(gz0, i) - h0;
            mi[1] = h2 - n2x;
            pl[2] = n1x - h1;
            mi[2] = h0 - el(gy0, i);
        }
        const float c0 = el(c[0], i);
        if (isnan(c0)) { /* general cell: rewritten by k_general32 after this launch */
            any_aux = true;
            continue;
        }
        const bool split = p.pmask[xx] | pyz;
        const float bn[3] = {c0, el(c[1], i), el(c[2], i)};
        if (!split) {
            float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
            if (on_src) {
                W[0] += (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 1, px0 + i));
                W[1] -= (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 0, px0 + i));
            }
#pragma unroll
            for (int cc = 0; cc < 3; cc++) set_el(out[cc], i, fmaf(sg * bn[cc], W[cc], el(out[cc], i)));
        } else {
            any_aux = true;
        }
    }
    /* elements that need their aux slot (split) or a record (general) */
    if (any_aux) {
        if (!qsplit) { /* a general (record) cell in an unsplit quad: rare */
#pragma unroll
            for (int cc = 0; cc < 3; cc++) aux[cc] = ld4(Fa + cc * n3 + l);
        }
        const int jy = s1 + j1, jz = s2 + j2;
        const float *tA = p.tab + (EF ? 2 : 0) * S, *tG = p.tab + (EF ? 3 : 1) * S;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int xx = x0 + i;
            const float c0 = el(c[0], i);
            if (isnan(c0)) continue;
            if (!(p.pmask[xx] | pyz)) continue;
            const float h0 = el(gh[0], i), h1 = el(gh[1], i), h2 = el(gh[2], i);
            float n1x, n2x;
            if (!EF) {
                n1x = i == 0 ? xn1 : el(gh[1], i - 1);
                n2x = i == 0 ? xn2 : el(gh[2], i - 1);
            } else {
                n1x = i == 3 ? xn1 : el(gh[1], i + 1);
                n2x = i == 3 ? xn2 : el(gh[2], i + 1);
            }
            float pl[3], mi[3];
            if (!EF) {
                pl[0] = h2 - el(gy2, i);
                mi[0] = el(gz1, i) - h1;
                pl[1] = h0 - el(gz0, i);
                mi[1] = n2x - h2;
                pl[2] = h1 - n1x;
                mi[2] = el(gy0, i) - h0;
            } else {
                pl[0] = el(gy2, i) - h2;
                mi[0] = h1 - el(gz1, i);
                pl[1] = el(gz0, i) - h0;
                mi[1] = h2 - n2x;
                pl[2] = n1x - h1;
                mi[2] = h0 - el(gy0, i);
            }
            const int jx[3] = {xx, jy, jz};
            const float bn[3] = {c0, el(c[1], i), el(c[2], i)};
#pragma unroll
            for (int cc = 0; cc < 3; cc++) {
                const int i1 = jx[(cc + 1) % 3], i2 = jx[(cc + 2) % 3];
                const float Ap = tA[i1], Bp = sg * bn[cc] * tG[i1];
                const float Am = tA[i2], Bm = sg * bn[cc] * tG[i2];
                const float m = el(aux[cc], i);
                const float pp = el(out[cc], i) - m; /* out still holds the old field here */
                const float np = fmaf(Bp, pl[cc], Ap * pp);
                const float nm = fmaf(Bm, mi[cc], Am * m);
                set_el(out[cc], i, np + nm);
                set_el(aux[cc], i, nm);
            }
        }
    }
#pragma unroll
    for (int cc = 0; cc < 3; cc++) st4(F + cc * n3 + l, out[cc]);
    if (any_aux) {
#pragma unroll
        for (int cc = 0; cc < 3; cc++) st4(Fa + cc * n3 + l, aux[cc]);
    }
    if (q >= 0) {
        /* split elements sample the total field, ordinary ones their field */
        st4(ring_at(p.d, g.pl, b, k, q, EF ? 2 : 0) + px0, out[0]);
        st4(ring_at(p.d, g.pl, b, k, q, EF ? 3 : 1) + px0, out[1]);
    }
}

/* MB: the register bound, as a minimum of resident 128-thread blocks per SM
 * (5: 96 registers, no spill; 6, 8: 80, 64 registers, more warps in flight
 * against a few spilled values) -- chosen by the autotuner */
template <bool EF, int MB>
__global__ void __launch_bounds__(128, MB) k_sweep32v(const P32 p, const int rel, const int z0)
{
    const int b = blockIdx.y % p.batch;
    const int xr = (blockIdx.x * 32 + threadIdx.x) * 4;
    const int j1 = (blockIdx.y / p.batch) * blockDim.y + threadIdx.y;
    sweep32v_quad<EF, false>(p, rel, b, j1, z0 + blockIdx.z, xr);
}

/* general cells of the vectorised sweeps: one thread per record cell, run
 * after k_sweep32v of the same field (the quads skipped them) */
template <bool EF, bool CG>
__device__ void general32_cell(const P32 &p, const int rel, const int b, const long long l)
{
    const Geo &g = p.g;
    const long long n3 = g.n3, bs = 3 * n3;
    const int j0 = (int)(l % g.L0), j1 = (int)((l / g.L0) % g.L1), j2 = (int)(l / g.pl);
    const float *__restrict__ cf = EF ? p.be : p.bh;
    float *F = (EF ? p.E : p.H) + b * bs, *Fa = (EF ? p.Ea : p.Ha) + b * bs;
    const float *G = (EF ? p.H : p.E) + b * bs, *Ga = (EF ? p.Ha : p.Ea) + b * bs;
    const float sg = EF ? 1.0f : -1.0f;
    const int k = *p.s.base + rel;
    const int px = j0 + g.L0 * j1;
    const int q = monitor_index(p.d, j2);
    const Rec32 r = (EF ? p.erec : p.hrec)[__float_as_int(cf[n3 + l])];
    const bool stable = r.kind == RK_STABLE;
    const Stn32 st = make_stn32(g, j0, j1, j2, EF && !stable);
    float main_out[3];
    if (r.kind == RK_FROZEN) {
        for (int c = 0; c < 3; c++) main_out[c] = F[c * n3 + l] - Fa[c * n3 + l];
    } else if (stable) {
        auto get = [&](int c, long long o) { return ldG<CG>(G + c * n3 + l + o) - ldG<CG>(Ga + c * n3 + l + o); };
        float pl[3], mi[3];
        curl32<false>(get, st, pl, mi);
        for (int c = 0; c < 3; c++) {
            const float W = pl[c] + mi[c];
            float x = Fa[c * n3 + l];
            float f = F[c * n3 + l] - x;
            f += 0.5f * x;
            x = fmaf(sg * r.B1[c], W, r.A1[c] * x);
            f += 0.5f * x;
            main_out[c] = f;
            F[c * n3 + l] = f + x;
            Fa[c * n3 + l] = x;
        }
    } else {
        auto get = [&](int c, long long o) { return ldG<CG>(G + c * n3 + l + o); };
        float pl[3], mi[3];
        curl32<EF>(get, st, pl, mi);
        if (r.kind == RK_N) {
            float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
            if (j2 == p.s.iI[b]) {
                W[0] += (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 1, px));
                W[1] -= (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 0, px));
            }
            for (int c = 0; c < 3; c++) {
                const float f = fmaf(sg * r.B0[c], W[c], r.A0[c] * F[c * n3 + l]);
                F[c * n3 + l] = f;
                main_out[c] = f;
            }
        } else {
            for (int c = 0; c < 3; c++) {
                const float m = Fa[c * n3 + l];
                const float pp = F[c * n3 + l] - m;
                const float np = fmaf(sg * r.B0[c], pl[c], r.A0[c] * pp);
                const float nm = fmaf(sg * r.B1[c], mi[c], r.A1[c] * m);
                F[c * n3 + l] = np + nm;
                Fa[c * n3 + l] = nm;
                main_out[c] = np + nm;
            }
        }
    }
    if (q >= 0) {
        ring_at(p.d, g.pl, b, k, q, EF ? 2 : 0)[px] = main_out[0];
        ring_at(p.d, g.pl, b, k, q, EF ? 3 : 1)[px] = main_out[1];
    }
}

template <bool EF>
__global__ void k_general32(const P32 p, const int rel, const int *cells, int ncells)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncells) return;
    general32_cell<EF, false>(p, rel, blockIdx.y, cells[i]);
}

/* ---------------------------------------------------------------------------
 * Groups: the vectorised H (E) sweep of every member plan in one launch.
 * Block i belongs to the member m with blk[m] <= i < blk[m+1]; inside it the
 * block decodes exactly as a k_sweep32v block (x block fastest, then row
 * block x excitation, then plane), so each member gets the same bits as
 * when it is stepped alone.  The member table lives in constant memory: a
 * block-uniform index into it is served by the constant cache, as kernel
 * parameters are, so a member's fields cost the sweep no extra registers.
 * One table per device: the host side runs one such group at a time.
 * ------------------------------------------------------------------------- */
__constant__ Group32 c_group;

template <bool EF>
__global__ void __launch_bounds__(128, 5) k_group32v(const int rel)
{
    int m = 0;
    while (m + 1 < c_group.n && (int)blockIdx.x >= c_group.blk[m + 1]) m++;
    const P32 &p = c_group.p[m];
    const int local = blockIdx.x - c_group.blk[m];
    const int nxb = (p.g.L0 / 4 + 31) / 32;
    const int nyb = ((p.g.L1 + c_group.by - 1) / c_group.by) * p.batch;
    const int xb = local % nxb, t = local / nxb;
    const int yb = t % nyb, z = t / nyb;
    const int b = yb % p.batch;
    const int j1 = (yb / p.batch) * blockDim.y + threadIdx.y;
    sweep32v_quad<EF, false>(p, rel, b, j1, z, (xb * 32 + threadIdx.x) * 4);
}

template <bool EF>
__global__ void k_group_general32(const int rel)
{
    const int *gb = EF ? c_group.gen_e : c_group.gen_h;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= gb[c_group.n]) return;
    int m = 0;
    while (m + 1 < c_group.n && i >= gb[m + 1]) m++;
    const int ng = EF ? c_group.negen[m] : c_group.nhgen[m];
    const int local = i - gb[m];
    general32_cell<EF, false>(c_group.p[m], rel, local / ng, (EF ? c_group.egen[m] : c_group.hgen[m])[local % ng]);
}

/* the member table for the steps that follow on stream st (from pinned host
 * memory, so that a captured graph reads it at each replay) */
void load_group32(const Group32 *host_pinned, cudaStream_t st)
{
    cudaMemcpyToSymbolAsync(c_group, host_pinned, sizeof(Group32), 0, cudaMemcpyHostToDevice, st);
}

void launch_group32v(const Group32 &gr, int rel, cudaStream_t st)
{
    const dim3 blk(32, gr.by, 1);
    k_group32v<false><<<gr.blk[gr.n], blk, 0, st>>>(rel);
    if (gr.gen_h[gr.n] > 0) k_group_general32<false><<<(gr.gen_h[gr.n] + 127) / 128, 128, 0, st>>>(rel);
    k_group32v<true><<<gr.blk[gr.n], blk, 0, st>>>(rel);
    if (gr.gen_e[gr.n] > 0) k_group_general32<true><<<(gr.gen_e[gr.n] + 127) / 128, 128, 0, st>>>(rel);
}

/* Fold `count` ring slots ending at step *base + rel_end into the FP64 DFT
 * accumulators (the reference's running DFT, FDTDsplitfieldMetal.c:318-328,
 * here on FP32 field samples): for each pixel, monitor plane, component and
 * frequency, acc += sum over the window of x_k * e^{i phi_k}, by compensated
 * (Kahan) summation in FP32.
 *   - each phase (FP64 in the schedule) is carried as a float pair hi + lo,
 *     hi = fl(phi), lo = fl(phi - hi): together exact to about 2^-48;
 *   - a term enters as y = fl(x*hi + (x*lo - c)), one rounding of the term
 *     less the running compensation c; then t = s + y, c = (t - s) - y, s = t.
 *     The window's error is then within about 3 units of 2^-24 of the sum of
 *     |terms| whatever the window length (a plain FP32 sum's bound grows with
 *     the number of terms);
 *   - the window's fl(s - c) is added to the FP64 accumulator.
 * A thread takes one pixel and one component of one plane and excitation,
 * its window's samples in registers, two frequencies at a time (independent
 * chains); the phases sit in shared memory frequency-major, so that a
 * frequency's samples are at fixed offsets.  Float to double goes by the IEEE
 * bit layout on the integer pipes (the FP64 pipe of this GPU is narrow; one
 * add per value is its only work here). */
constexpr int RING_MAX = 32;

/* one Kahan step: s the sum, n the negated compensation, term x * (hi + lo);
 * the _rn intrinsics keep every operation separately rounded (no contraction
 * may merge or reorder them) */
__device__ __forceinline__ void kahan_term(float x, float hi, float lo, float &s, float &n)
{
    const float y = __fmaf_rn(x, hi, __fmaf_rn(x, lo, n));
    const float t = __fadd_rn(s, y);
    n = __fsub_rn(y, __fsub_rn(t, s));
    s = t;
}

/* float -> double by the bit layout: sign, exponent rebiased (127 -> 1023),
 * mantissa shifted into place; zero and subnormal floats (below 2^-126) give
 * zero, infinities and NaNs keep their class */
__device__ __forceinline__ double widen(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned ed = e == 0xffu ? 0x7ffu : e + 896u;
    const unsigned hi = (u & 0x80000000u) | (ed << 20) | ((u & 0x7fffffu) >> 3);
    const unsigned lo = u << 29;
    return e == 0u ? 0.0 : __hiloint2double((int)hi, (int)lo);
}

/* CMAX: the window length rounded up to a multiple of 8; FULL: the window is
 * the whole ring (CMAX = RING_MAX samples, no per-sample predicate).  A
 * shorter window at the end of a run skips the samples past its length, so
 * its cost follows its length; only a window of exactly RING_MAX samples may
 * take FULL (the phase table in shared memory holds count_rt samples). */
template <int CMAX, bool FULL>
__global__ void __launch_bounds__(128, 6) k_flush32(const P32 p, const int rel_end, const int count_rt)
{
    /* [nfreq][count] {hi re, hi im, lo re, lo im} of this block's half (H or E
     * phases) */
    extern __shared__ float4 sph[];
    static_assert(!FULL || CMAX == RING_MAX, "a full window is the whole ring");
    const int count = FULL ? RING_MAX : count_rt;
    const Dft &d = p.d;
    const int k0 = *p.s.base + rel_end - count;
    const int qv = blockIdx.y, b = blockIdx.z;
    const int q = qv >> 2, v = qv & 3, half = v >> 1;
    const int nph = count * d.nfreq;
    const float4 *ph4 = reinterpret_cast<const float4 *>(d.xphase32 ? d.xphase32 : d.phase32);
    for (int i = threadIdx.x; i < nph; i += blockDim.x) {
        const int f = i / count, s = i % count;
        sph[i] = d.xphase32 ? ph4[half] : ph4[((long long)(k0 + s) * d.nfreq + f) * 2 + half];
    }
    __syncthreads();
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= p.g.pl) return;
    float x[CMAX];
#pragma unroll
    for (int s = 0; s < CMAX; s++) x[s] = (s < count) ? ring_at(d, p.g.pl, b, k0 + s, q, v)[px] : 0.0f;
    double *acc = d.acc + 2 * (((((long long)b * d.nfreq) * d.nq + q) * 4 + v) * p.g.pl + px);
    const long long fstride = 2 * (long long)d.nq * 4 * p.g.pl; /* doubles from one frequency to the next */
    int f = 0;
    for (; f + 1 < d.nfreq; f += 2) {
        const float4 *pa = sph + f * count, *pb = pa + count;
        float sa = 0.f, na = 0.f, sai = 0.f, nai = 0.f, sb = 0.f, nb = 0.f, sbi = 0.f, nbi = 0.f;
#pragma unroll
        for (int s = 0; s < CMAX; s++) {
            if (FULL || s < count) {
                const float4 ha = pa[s], hb = pb[s];
                kahan_term(x[s], ha.x, ha.z, sa, na);
                kahan_term(x[s], ha.y, ha.w, sai, nai);
                kahan_term(x[s], hb.x, hb.z, sb, nb);
                kahan_term(x[s], hb.y, hb.w, sbi, nbi);
            }
        }
        double *a = acc + f * fstride;
        a[0] += widen(__fadd_rn(sa, na));
        a[1] += widen(__fadd_rn(sai, nai));
        a[fstride] += widen(__fadd_rn(sb, nb));
        a[fstride + 1] += widen(__fadd_rn(sbi, nbi));
    }
    if (f < d.nfreq) {
        const float4 *pa = sph + f * count;
        float sa = 0.f, na = 0.f, sai = 0.f, nai = 0.f;
#pragma unroll
        for (int s = 0; s < CMAX; s++) {
            if (FULL || s < count) {
                const float4 ha = pa[s];
                kahan_term(x[s], ha.x, ha.z, sa, na);
                kahan_term(x[s], ha.y, ha.w, sai, nai);
            }
        }
        double *a = acc + f * fstride;
        a[0] += widen(__fadd_rn(sa, na));
        a[1] += widen(__fadd_rn(sai, nai));
    }
}

/* Sweeps over the planes z0 <= z < z1 (the whole grid: 0, L2). */
void launch_h32(const P32 &p, int rel, int by, int z0, int z1, cudaStream_t st)
{
    dim3 blk(32, by, 1), grd((p.g.L0 + 31) / 32, ((p.g.L1 + by - 1) / by) * p.batch, z1 - z0);
    k_sweep32<false><<<grd, blk, 0, st>>>(p, rel, z0);
}

void launch_e32(const P32 &p, int rel, int by, int z0, int z1, cudaStream_t st)
{
    dim3 blk(32, by, 1), grd((p.g.L0 + 31) / 32, ((p.g.L1 + by - 1) / by) * p.batch, z1 - z0);
    k_sweep32<true><<<grd, blk, 0, st>>>(p, rel, z0);
}

/* gcells / ngh: the general cells of those planes */
/* Two z-planes per thread: the loads of both quads leave before either is
 * computed, so a warp keeps twice the bytes in flight at the same occupancy
 * (the single-plane sweep is latency-bound).  Same updates, same bits.  MB as
 * for k_sweep32v (4: 128 registers). */
template <bool EF, int MB>
__global__ void __launch_bounds__(128, MB) k_sweep32v2(const P32 p, const int rel, const int z0, const int z1)
{
    const int b = blockIdx.y % p.batch;
    const int xr = (blockIdx.x * 32 + threadIdx.x) * 4;
    const int j1 = (blockIdx.y / p.batch) * blockDim.y + threadIdx.y;
    const int za = z0 + 2 * blockIdx.z;
    const bool two = za + 1 < z1;
    QIn qa, qb;
    if (!quad_load<EF, false>(p, b, j1, za, xr, qa)) return;
    if (two) quad_load<EF, false>(p, b, j1, za + 1, xr, qb);
    quad_compute<EF>(p, rel, b, j1, za, qa);
    if (two) quad_compute<EF>(p, rel, b, j1, za + 1, qb);
}

template <bool EF>
static void launch_sweep32v(const P32 &p, int rel, int by, int mb, int z0, int z1, cudaStream_t st)
{
    dim3 blk(32, by, 1), grd((p.g.L0 / 4 + 31) / 32, ((p.g.L1 + by - 1) / by) * p.batch, z1 - z0);
    if (mb < 0) { /* two planes per thread: -mb = register bound */
        grd.z = (z1 - z0 + 1) / 2;
        if (mb == -3) k_sweep32v2<EF, 3><<<grd, blk, 0, st>>>(p, rel, z0, z1);
        else k_sweep32v2<EF, 4><<<grd, blk, 0, st>>>(p, rel, z0, z1);
        return;
    }
    if (mb >= 8) k_sweep32v<EF, 8><<<grd, blk, 0, st>>>(p, rel, z0);
    else if (mb == 6) k_sweep32v<EF, 6><<<grd, blk, 0, st>>>(p, rel, z0);
    else k_sweep32v<EF, 5><<<grd, blk, 0, st>>>(p, rel, z0);
}

void launch_h32v(const P32 &p, int rel, int by, int mb, int z0, int z1, const int *gcells, int ngh,
                 cudaStream_t st)
{
    launch_sweep32v<false>(p, rel, by, mb, z0, z1, st);
    if (ngh > 0) k_general32<false><<<dim3((ngh + 127) / 128, p.batch), 128, 0, st>>>(p, rel, gcells, ngh);
}

void launch_e32v(const P32 &p, int rel, int by, int mb, int z0, int z1, const int *gcells, int nge,
                 cudaStream_t st)
{
    launch_sweep32v<true>(p, rel, by, mb, z0, z1, st);
    if (nge > 0) k_general32<true><<<dim3((nge + 127) / 128, p.batch), 128, 0, st>>>(p, rel, gcells, nge);
}

void launch_flush32(const P32 &p, int rel_end, int count, cudaStream_t st)
{
    /* callers flush at least once every RING_MAX steps (the ring's length) */
    if (p.d.nfreq <= 0 || p.d.nq <= 0 || count <= 0 || count > RING_MAX) return;
    dim3 blk(128), grd((p.g.pl + 127) / 128, p.d.nq * 4, p.batch);
    const size_t sm = sizeof(float4) * (size_t)count * p.d.nfreq;
    static_assert(RING_MAX == 32, "flush instantiations: windows rounded up to 8, 16, 24, 32");
    const int cmax = (count + 7) / 8 * 8;
    const void *fn = count == RING_MAX ? (const void *)k_flush32<32, true>
                     : cmax == 8       ? (const void *)k_flush32<8, false>
                     : cmax == 16      ? (const void *)k_flush32<16, false>
                     : cmax == 24      ? (const void *)k_flush32<24, false>
                                       : (const void *)k_flush32<32, false>;
    if (sm > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    void *args[] = {(void *)&p, (void *)&rel_end, (void *)&count};
    cudaLaunchKernel(fn, grd, blk, args, sm, st);
}

} // namespace smat
