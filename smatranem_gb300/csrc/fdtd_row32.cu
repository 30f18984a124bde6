/*
 * FP32 split-field FDTD: one fused launch per Yee step over whole x rows
 * (launch form 6).
 *
 * Same update as the two FP32 sweeps of fdtd_f32.cu (the reference main_calc,
 * FDTDcalc/FDTDsplitfieldMetal.c:242-329, in total-field form), with the same
 * floating point expressions, so the results are bit-identical to them.  For
 * plans with L0 % 4 == 0 (record cells -- lossy and PEC ordinary cells, lossy
 * split cells, metal cells -- run a compile-time variant, REC; the
 * stable-form E update of metal cells and the monitor samples of metal cells
 * run in a second, small launch after the step, k_row_metal).
 *
 *   - a CTA owns TY whole x rows (y0 .. y0+TY-1) of one excitation and marches
 *     along z through a range of planes [z0, z1).  At stage z it computes
 *     H_new(z) on its rows plus one halo row (y0+TY, recomputed, never stored),
 *     then E_new(z-1) on its rows, which needs H_new of planes z-1 and z: of
 *     plane z on its own column from registers, of plane z-1 (its own cells,
 *     the row above, the quad to the right) from a two-plane ring in shared
 *     memory.  One barrier a stage.
 *   - a thread owns one quad (four x-cells, float4) of one row for the whole
 *     march.  Each field value is read once and written once per step (48 B
 *     per cell and excitation, plus the coefficient stream and the aux slots
 *     of split cells): the compulsory traffic of a step, where the two sweeps
 *     move 72 B.  Quads whose x index lies in a PML take the first threads, so
 *     that the other warps run the ordinary update without the split branch.
 *   - the inputs of the next plane are in flight while the current one is
 *     computed: cp.async copies into shared memory of the next plane's E
 *     (double-buffered: the neighbouring threads read it for the y-1 and x-1
 *     terms; the first row also stages the E row above the tile), of the
 *     thread's own bh, H, H aux of the next plane and be, E aux of this plane
 *     (one slot each, refilled right after use), so the stage barrier does not
 *     wait on a DRAM round trip and no registers are held by loads in flight.
 *   - whole rows: the x wrap is inside the row.
 *   - fields are double-buffered (read the current set, write the other), so
 *     the halo reads of a neighbouring CTA never see an advanced value.
 *   - the plane z1 closing a range: H_new(z1) is recomputed, not stored; at
 *     z1 = L2 it is iBc_z * H_new(0), which is what the sweeps read through the
 *     wrapped z boundary (:334, :355); a wrapped halo row likewise holds
 *     iBc_y * H_new(row 0).  Ranges are independent: fixed z chunks, one per
 *     CTA, or persistent CTAs marching whole row tiles in rounds.
 */
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"
#include "host_internal.h"
#include "smatran_fdtd.h"

namespace smat {
namespace {

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

/* 16-byte global -> shared copy that bypasses L1 (each staged value is read
 * from shared memory only) */
__device__ __forceinline__ void cpa16(float4 *dst, const float *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cpa_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
/* all but this thread's two most recent groups complete */
__device__ __forceinline__ void cpa_wait2() { asm volatile("cp.async.wait_group 2;\n" ::: "memory"); }

/* the source sheet of step k (the sweeps' expression) */
__device__ __forceinline__ double row_sheet(const Src &s, int pl, int b, int k, bool efield, int v, int p)
{
    if (s.xsrc) return s.xsrc[(efield ? 2 * pl : 0) + v + 2 * p];
    const double *sc = s.sched + 6 * (long long)k + (efield ? 0 : 3);
    const double *w = s.inc + (long long)b * 8 * pl + (efield ? 4 * pl : 0) + 2 * (v + 2 * p);
    return sc[0] * (sc[1] * w[0] + sc[2] * w[1]);
}

__device__ __forceinline__ int row_monitor(const Dft &d, int j2)
{
    int q = -1;
#pragma unroll
    for (int i = 0; i < MAX_PLANES; i++)
        if (i < d.nq && d.planes[i] == j2) q = i;
    return q;
}

__device__ __forceinline__ float *row_ring(const Dft &d, int pl, int b, int k, int q, int v)
{
    const int slot = k % d.ringK;
    return d.ring + ((((long long)b * d.ringK + slot) * d.nq + q) * 4 + v) * (long long)pl;
}

/* The 1-D split-PML factors A(sigma), G(sigma) of one field at a quad's four
 * x indices, its row and its plane, and the PML bits of the four x indices:
 * loaded once per thread (the plane's once per stage) instead of per element. */
struct QuadTab {
    float ax[4], gx[4];
    float ay, gy, az, gz;
    unsigned xm;
};

/* A metal cell's stable-form or frozen component in the march: the aux slot
 * from the old set (it is staged only where the quad is split; the caller
 * stores the aux slots of every quad with a record cell) into ta; an H
 * stable-form component updates t and ta from the backward curl of E's main
 * slot (E - Ea, old set, from global memory), as the sweeps do; an E
 * stable-form component is left for k_row_metal after the step, and a frozen
 * one keeps its values.  Out of line from the record path (metal cells are
 * rarer still). */
template <bool EF>
__device__ __noinline__ void row_metal_record(const P32 &p, const int b, const int px, const int j2, const Rec32 &r,
                                              float *t, float *ta)
{
    const Geo &g = p.g;
    const long long n3 = g.n3, bs = 3 * n3, l = px + (long long)g.pl * j2;
    const float *Fa = (EF ? p.Ea : p.Ha) + b * bs;
    float x[3] = {Fa[l], Fa[n3 + l], Fa[2 * n3 + l]};
    if (!EF && r.kind == RK_STABLE) {
        /* the stable form differentiates the MAIN slot of the other field */
        const float sg = -1.0f;
        const float *G = p.E + b * bs, *Ga = p.Ea + b * bs;
        const Stn32 st = make_stn32(g, px % g.L0, px / g.L0, j2, false);
        auto get = [&](int c, long long o) { return G[c * n3 + l + o] - Ga[c * n3 + l + o]; };
        float ps[3], ms[3];
        curl32<false>(get, st, ps, ms);
        for (int c = 0; c < 3; c++) {
            const float W = ps[c] + ms[c];
            float xc = x[c];
            float f = t[c] - xc;
            f += 0.5f * xc;
            xc = fmaf(sg * r.B1[c], W, r.A1[c] * xc);
            f += 0.5f * xc;
            t[c] = f + xc;
            x[c] = xc;
        }
    }
    for (int c = 0; c < 3; c++) ta[c] = x[c];
}

/* A record cell -- an ordinary ('n') cell that is lossy or PEC, a split cell
 * with lossy media (RK_A), or a metal cell's stable-form or frozen component
 * (row_metal_record) -- updated as the sweeps' general-cell path does
 * (fdtd_f32.cu, general32_cell); t is the cell's total field, ta its aux
 * slot, both updated in place; pl, mi the half curls of the other field's
 * total.  Out of line: record cells are rare and must not cost the quads
 * registers. */
template <bool EF>
__device__ __noinline__ void row_record(const P32 &p, const int k, const int b, const bool on_src, const int px,
                                        const int j2, const int ridx, const float *pl, const float *mi, float *t,
                                        float *ta)
{
    const Geo &g = p.g;
    const float sg = EF ? 1.0f : -1.0f;
    const Rec32 r = (EF ? p.erec : p.hrec)[ridx];
    if (r.kind == RK_A) { /* the two halves of a split cell, record coefficients */
        for (int c = 0; c < 3; c++) {
            const float m = ta[c];
            const float pp = t[c] - m;
            const float np = fmaf(sg * r.B0[c], pl[c], r.A0[c] * pp);
            const float nm = fmaf(sg * r.B1[c], mi[c], r.A1[c] * m);
            t[c] = np + nm;
            ta[c] = nm;
        }
        return;
    }
    if (r.kind == RK_STABLE || r.kind == RK_FROZEN) {
        row_metal_record<EF>(p, b, px, j2, r, t, ta);
        return;
    }
    float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
    if (on_src) {
        W[0] += (float)(p.s.sgn[b] * row_sheet(p.s, g.pl, b, k, !EF, 1, px));
        W[1] -= (float)(p.s.sgn[b] * row_sheet(p.s, g.pl, b, k, !EF, 0, px));
    }
    for (int c = 0; c < 3; c++) t[c] = fmaf(sg * r.B0[c], W[c], r.A0[c] * t[c]);
}

/* The update of one quad -- H (EF = false) or E (EF = true) of cells x0..x0+3
 * of row j1, plane j2 -- in place in out (total field) and aux (split cells),
 * from the other field at the cells (gh), its y and z neighbours (gy0, gy2:
 * components 0 and 2 one row away; gz0, gz1: components 0 and 1 one plane
 * away, both already scaled by the boundary factor) and the outer x neighbour
 * of the quad (xn1, xn2: components 1 and 2).  The expressions of the
 * vectorised sweep (fdtd_f32.cu), element by element. */
template <bool EF, bool REC>
__device__ __forceinline__ void row_quad(const P32 &p, const int k, const int b, const int j1, const int j2,
                                         const int x0, const bool on_src, const QuadTab &tq, const float4 c[3],
                                         float4 out[3], const float4 gh[3], float4 aux[3], const float4 gy0,
                                         const float4 gy2, const float4 gz0, const float4 gz1, const float xn1,
                                         const float xn2, const bool pyz)
{
    const Geo &g = p.g;
    const float sg = EF ? 1.0f : -1.0f;
    const int px0 = x0 + g.L0 * j1;
#pragma unroll
    for (int i = 0; i < 4; i++) {
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
        if (!EF) { /* backward differences */
            pl[0] = h2 - el(gy2, i);
            mi[0] = el(gz1, i) - h1;
            pl[1] = h0 - el(gz0, i);
            mi[1] = n2x - h2;
            pl[2] = h1 - n1x;
            mi[2] = el(gy0, i) - h0;
        } else { /* forward differences */
            pl[0] = el(gy2, i) - h2;
            mi[0] = h1 - el(gz1, i);
            pl[1] = el(gz0, i) - h0;
            mi[1] = h2 - n2x;
            pl[2] = n1x - h1;
            mi[2] = h0 - el(gy0, i);
        }
        const float bn[3] = {el(c[0], i), el(c[1], i), el(c[2], i)};
        if (REC && isnan(bn[0])) { /* a record cell (marked by NaN in its first coefficient) */
            float t[3] = {el(out[0], i), el(out[1], i), el(out[2], i)};
            float ta[3] = {el(aux[0], i), el(aux[1], i), el(aux[2], i)}; /* staged where the quad is split */
            row_record<EF>(p, k, b, on_src, px0 + i, j2, __float_as_int(bn[1]), pl, mi, t, ta);
#pragma unroll
            for (int cc = 0; cc < 3; cc++) {
                set_el(out[cc], i, t[cc]);
                set_el(aux[cc], i, ta[cc]);
            }
        } else if (!(((tq.xm >> i) & 1u) | pyz)) {
            float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
            if (on_src) {
                W[0] += (float)(p.s.sgn[b] * row_sheet(p.s, g.pl, b, k, !EF, 1, px0 + i));
                W[1] -= (float)(p.s.sgn[b] * row_sheet(p.s, g.pl, b, k, !EF, 0, px0 + i));
            }
#pragma unroll
            for (int cc = 0; cc < 3; cc++) set_el(out[cc], i, fmaf(sg * bn[cc], W[cc], el(out[cc], i)));
        } else {
            /* the factors of axis a: x (0), y (1), z (2) */
            const float tA[3] = {tq.ax[i], tq.ay, tq.az}, tG[3] = {tq.gx[i], tq.gy, tq.gz};
#pragma unroll
            for (int cc = 0; cc < 3; cc++) {
                const int i1 = (cc + 1) % 3, i2 = (cc + 2) % 3;
                const float Ap = tA[i1], Bp = sg * bn[cc] * tG[i1];
                const float Am = tA[i2], Bm = sg * bn[cc] * tG[i2];
                const float m = el(aux[cc], i);
                const float pp = el(out[cc], i) - m;
                const float np = fmaf(Bp, pl[cc], Ap * pp);
                const float nm = fmaf(Bm, mi[cc], Am * m);
                set_el(out[cc], i, np + nm);
                set_el(aux[cc], i, nm);
            }
        }
    }
}

/* Shared memory (float4 units):
 *   es  [2][3][NC]       staged E of a plane (read by the neighbouring threads:
 *                        double-buffered, slot z & 1)
 *   ph  [3][3][NC]       staged bh, H, H aux of the next plane (read by their
 *                        own thread only: one slot, refilled right after use)
 *   pe  [2][3][NC]       staged be, E aux of the plane whose E update is next
 *   top [2][2][NQ]       E components 0 and 2 of the row above the tile
 *   hs  [2][TY+1][3][NQ] H_new of the last two planes (the halo row last)
 *   the plane table of the plane range (PlaneInfo, 2 float4 a plane)
 * with NC = (TY+1) * NQ quads, quad q of tile row r at r * NQ + q.
 * cp.async groups, three a stage, in this order: E of plane z+1 (G1), bh/H/aux
 * of plane z+1 (G2, after the H update), be/E aux of plane z (G3, after the E
 * update).  Each wait leaves the two most recent groups in flight. */
size_t row_smem_f4(int L0, int ty, int zc)
{
    const size_t nq = L0 / 4, nc = nq * (ty + 1);
    return 21 * nc + 4 * nq + 6 * nc + 2 * (size_t)(zc + 1);
}

/* a 16-byte shared-memory load kept whole (lanes reading consecutive quads
 * then access consecutive 16-byte words: no bank conflicts) */
__device__ __forceinline__ float4 lds4(const float4 *a)
{
    float4 v;
    const unsigned s = (unsigned)__cvta_generic_to_shared(a);
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];\n"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(s)
                 : "memory");
    return v;
}

/* per plane of a range: the 1-D split-PML factors of its z index (H: A, G;
 * E: A, G), whether it lies in a PML and its monitor index (or -1) */
struct PlaneInfo {
    float ah, gh, ae, ge;
    int pm, q, pad0, pad1;
};

/* The march of one CTA through the pieces next(yt, z0, z1) gives -- rows
 * yt*TY .. of excitation b through planes [z0, z1) -- by the whole CTA (every
 * thread sees the same pieces).  The per-thread setup (quad, split factors)
 * is done once.  At the end of each piece every shared-memory read of it has
 * passed a barrier, so the next piece (of this plan or, in a group, of
 * another) may restage at once. */
template <bool REC, class Next>
__device__ __forceinline__ void row_march(const Row32 &r, const int rel, const int b, Next &&next)
{
    extern __shared__ float4 sm4[];
    const P32 &p = r.p;
    const Geo &g = p.g;
    const int L0 = g.L0, L1 = g.L1, L2 = g.L2, NQ = L0 >> 2, TY = r.ty, NR = TY + 1;
    const int NC = NR * NQ, T = blockDim.x;
    const long long n3 = g.n3, bs = 3 * n3, pl = g.pl;
    const int s1 = L0, s2 = L0 + L1;
    const int tid = threadIdx.x;
    float4 *const es = sm4, *const ph = sm4 + 6 * NC, *const pe = sm4 + 15 * NC, *const top = sm4 + 21 * NC,
                  *const hs = top + 4 * NQ;
    PlaneInfo *const pinfo = reinterpret_cast<PlaneInfo *>(hs + 6 * NC); /* planes z0 .. z1 */
#define ES(s, c) es[((s) * 3 + (c)) * NC]
#define PH(f, c) ph[((f) * 3 + (c)) * NC]
#define PE(f, c) pe[((f) * 3 + (c)) * NC]
#define TOP(s, c) top[((s) * 2 + (c)) * NQ]
#define HS(z, row, c) hs[((((z) & 1) * NR + (row)) * 3 + (c)) * NQ]

    /* this thread's quad: the quads of the tile's rows whose x index lies in
     * a PML (split cells) take the first threads, row by row, the others the
     * rest, so that whole warps run the ordinary update with no split-cell
     * branch (in x order within each group: r.qorder) */
    const int nqp = r.nqp, nqi = NQ - nqp;
    /* the thread's place in that order: with r.worder the last two warps
     * (mostly the halo row's quads, which skip the E update) trade places
     * with the two before them, so that they share the SM sub-partitions of
     * warps 0 and 1 (the split quads); warps go to the four sub-partitions
     * by warp index mod 4 */
    int qt = tid;
    if (r.worder && (T & 127) == 0 && T >= 256) {
        const int w = qt >> 5, W = T >> 5;
        if (w >= W - 4) qt += w < W - 2 ? 64 : -64;
    }
    int ry = TY, xq = NQ - 1;
    const bool xlive = qt < NC; /* threads past the tile's quads idle */
    if (qt < NR * nqp) {
        ry = qt / nqp;
        xq = r.qorder[qt % nqp];
    } else if (xlive) {
        const int u = qt - NR * nqp;
        ry = u / nqi;
        xq = r.qorder[nqp + u % nqi];
    }
    const int sid = ry * NQ + xq; /* its staging slot */
    const int xs = xq;
    const int x0 = 4 * xs;
    const bool halo = ry == TY;
    const int k = *p.s.base + rel;
    const float fxm = x0 == 0 ? (float)g.bc[0] : 1.0f; /* x-1 neighbour wrapped with iBc_x */
    const int xl = x0 == 0 ? NQ - 1 : xs - 1;
    const bool xe1 = x0 + 4 == L0;
    const float fxp = xe1 ? (float)g.bc[0] : 1.0f; /* x+1 neighbour of the E update */
    const int xqn = xe1 ? 0 : xs + 1;
    const int S = L0 + L1 + L2;
    QuadTab th, te; /* split-PML factors of the H and the E update */
    th.xm = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        th.xm |= (unsigned)(p.pmask[x0 + i] != 0) << i;
        th.ax[i] = p.tab[x0 + i];
        th.gx[i] = p.tab[S + x0 + i];
        te.ax[i] = p.tab[2 * S + x0 + i];
        te.gx[i] = p.tab[3 * S + x0 + i];
    }
    te.xm = th.xm;
    const bool pmx = th.xm != 0;
    const int iIb = p.s.iI[b]; /* the excitation's source plane */

    for (;;) {
        int yt, z0, z1;
        if (!next(yt, z0, z1)) break;
        const int Y0 = yt * TY, h = min(TY, L1 - Y0);
        /* this thread's row: own rows 0..h-1, rows h..TY-1 idle (a partial last
         * tile), row TY the halo row y0+h */
        const bool own = !halo && ry < h && xlive;
        const bool act = own || (halo && xlive); /* stages and computes H_new */
        int gy = halo ? Y0 + h : min(Y0 + ry, L1 - 1);
        float fyw = 1.0f; /* the halo row wrapped to row 0 holds iBc_y * H_new */
        if (gy == L1) {
            gy = 0;
            fyw = (float)g.bc[1];
        }
        const int rown = ry + 1 == h ? TY : ry + 1; /* H_new row of the y+1 neighbour */
        const int yb = halo ? h - 1 : ry - 1;       /* staged E row of the y-1 neighbour (ry = 0: top) */
        const long long lr = x0 + (long long)L0 * gy + b * bs;
        const int px0 = x0 + L0 * gy;
        const float fy = gy == 0 ? (float)g.bc[1] : 1.0f; /* y-1 neighbour wrapped with iBc_y */
        const int gtop = Y0 == 0 ? L1 - 1 : Y0 - 1;         /* the row above the tile */
        const bool pmy = p.pmask[s1 + gy];
        th.ay = p.tab[s1 + gy];
        th.gy = p.tab[S + s1 + gy];
        te.ay = p.tab[2 * S + s1 + gy];
        te.gy = p.tab[3 * S + s1 + gy];

        /* G1: E of stage z (plane z, or 0 for z = L2) and the row above */
        auto stage_e_old = [&](int z) {
            const int zr = z == L2 ? 0 : z, s = z & 1;
            const long long l = lr + pl * zr;
#pragma unroll
            for (int i = 0; i < 3; i++) cpa16(&ES(s, i) + sid, p.E + i * n3 + l);
            if (ry == 0) {
                const long long lt = x0 + (long long)L0 * gtop + b * bs + pl * zr;
                cpa16(&TOP(s, 0) + xq, p.E + lt);
                cpa16(&TOP(s, 1) + xq, p.E + 2 * n3 + lt);
            }
        };
        /* G2: bh, H, H aux of stage z */
        auto stage_h = [&](int z) {
            const int zr = z == L2 ? 0 : z;
            const long long l = lr + pl * zr, lc = l - b * bs;
#pragma unroll
            for (int i = 0; i < 3; i++) {
                cpa16(&PH(0, i) + sid, p.bh + i * n3 + lc);
                cpa16(&PH(1, i) + sid, p.H + i * n3 + l);
            }
            if (pmy | pinfo[z - z0].pm | pmx) {
#pragma unroll
                for (int i = 0; i < 3; i++) cpa16(&PH(2, i) + sid, p.Ha + i * n3 + l);
            }
        };
        /* G3: be, E aux of plane z (its E update runs at stage z + 1) */
        auto stage_e = [&](int z) {
            const long long l = lr + pl * z, lc = l - b * bs;
#pragma unroll
            for (int i = 0; i < 3; i++) cpa16(&PE(0, i) + sid, p.be + i * n3 + lc);
            if (pmy | pinfo[z - z0].pm | pmx) {
#pragma unroll
                for (int i = 0; i < 3; i++) cpa16(&PE(1, i) + sid, p.Ea + i * n3 + l);
            }
        };

        /* the plane table of the chunk (z1 = L2 is plane 0) */
        for (int j = tid; j <= z1 - z0; j += T) {
            const int zz = z0 + j == L2 ? 0 : z0 + j;
            PlaneInfo pi;
            pi.ah = p.tab[s2 + zz];
            pi.gh = p.tab[S + s2 + zz];
            pi.ae = p.tab[2 * S + s2 + zz];
            pi.ge = p.tab[3 * S + s2 + zz];
            pi.pm = p.pmask[s2 + zz] != 0;
            pi.q = row_monitor(p.d, zz);
            pi.pad0 = pi.pad1 = 0;
            pinfo[j] = pi;
        }
        __syncthreads();

        /* E_old(z0-1), components 0 and 1 (the z-1 neighbour of H_new(z0)), and
         * the inputs of the first stage */
        float4 Ep[3];
        Ep[2] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (act) {
            int zp = z0 - 1;
            float fz = 1.0f;
            if (zp < 0) {
                zp = L2 - 1;
                fz = (float)g.bc[2];
            }
            const long long l = lr + pl * zp;
            Ep[0] = scale4(ld4(p.E + l), fz);
            Ep[1] = scale4(ld4(p.E + n3 + l), fz);
            stage_e_old(z0);
            stage_h(z0);
        }
        cpa_commit();
        cpa_wait_all();
        __syncthreads();

        for (int z = z0; z <= z1; z++) {
            const bool wz = z == L2; /* the closing plane wraps to 0 */
            const int zr = wz ? 0 : z, s = z & 1;
            const float fzw = wz ? (float)g.bc[2] : 1.0f;
            /* G1: the next plane's E leaves now (its slot was last read before
             * the previous barrier) */
            if (act && z < z1) stage_e_old(z + 1);
            cpa_commit();
            float4 o[3], e[3];
            if (act) {
                /* this thread's bh, H, aux of plane z (the previous stage's G2) */
                cpa_wait2();
                const PlaneInfo zi = pinfo[z - z0];
                const bool pyz = pmy | zi.pm;
                const bool qs = pyz | pmx;
                float4 c[3], a[3];
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    c[i] = (&PH(0, i))[sid];
                    o[i] = (&PH(1, i))[sid];
                    e[i] = (&ES(s, i))[sid];
                }
                if (qs) {
#pragma unroll
                    for (int i = 0; i < 3; i++) a[i] = (&PH(2, i))[sid];
                } else if (REC) { /* record cells read the aux values; none is split here */
#pragma unroll
                    for (int i = 0; i < 3; i++) a[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
                float4 gy0, gy2;
                if (ry == 0) {
                    gy0 = scale4((&TOP(s, 0))[xq], fy);
                    gy2 = scale4((&TOP(s, 1))[xq], fy);
                } else {
                    gy0 = scale4((&ES(s, 0))[yb * NQ + xs], fy);
                    gy2 = scale4((&ES(s, 2))[yb * NQ + xs], fy);
                }
                /* x-1 neighbour: the staged E of the quad to the left */
                const float xn1 = fxm * lds4(&ES(s, 1) + ry * NQ + xl).w, xn2 = fxm * lds4(&ES(s, 2) + ry * NQ + xl).w;
                const float4 gz0 = scale4(Ep[0], fzw), gz1 = scale4(Ep[1], fzw);
                th.az = zi.ah;
                th.gz = zi.gh;
                /* the aux slots leave for split quads and quads with a record
                 * cell (a metal cell's aux slot; zeros elsewhere) */
                const bool qa = qs || (REC && (isnan(c[0].x) | isnan(c[0].y) | isnan(c[0].z) | isnan(c[0].w)));
                row_quad<false, REC>(p, k, b, gy, zr, x0, zr == iIb, th, c, o, e, a, gy0, gy2, gz0, gz1, xn1, xn2, pyz);
                /* the private slot is free: plane z+1's bh, H, aux leave */
                if (z < z1) stage_h(z + 1);
                const long long l = lr + pl * zr;
                if (own && z < z1) {
#pragma unroll
                    for (int i = 0; i < 3; i++) st4(r.Hn + i * n3 + l, o[i]);
                    if (qa) {
#pragma unroll
                        for (int i = 0; i < 3; i++) st4(r.Han + i * n3 + l, a[i]);
                    }
                    const int q = zi.q;
                    if (q >= 0) {
                        st4(row_ring(p.d, g.pl, b, k, q, 0) + px0, o[0]);
                        st4(row_ring(p.d, g.pl, b, k, q, 1) + px0, o[1]);
                    }
                }
#pragma unroll
                for (int i = 0; i < 3; i++) (&HS(z, ry, i))[xs] = scale4(o[i], fyw);
            }
            cpa_commit(); /* G2 */
            if (own && z > z0) {
                /* this thread's be, E aux of plane z-1 (the previous stage's G3) */
                cpa_wait2();
                const int ze = z - 1;
                const long long le = lr + pl * ze;
                const PlaneInfo zi = pinfo[ze - z0];
                const bool pyze = pmy | zi.pm;
                const bool qse = pyze | pmx;
                float4 ce[3], ae[3];
#pragma unroll
                for (int i = 0; i < 3; i++) ce[i] = (&PE(0, i))[sid];
                if (qse) {
#pragma unroll
                    for (int i = 0; i < 3; i++) ae[i] = (&PE(1, i))[sid];
                } else if (REC) {
#pragma unroll
                    for (int i = 0; i < 3; i++) ae[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
                /* H_new of plane z-1 (own quad, row above, quad to the right) from
                 * shared memory, of plane z from registers */
                const float4 hp[3] = {(&HS(ze, ry, 0))[xs], (&HS(ze, ry, 1))[xs], (&HS(ze, ry, 2))[xs]};
                const float4 ey0 = (&HS(ze, rown, 0))[xs], ey2 = (&HS(ze, rown, 2))[xs];
                const float4 ez0 = scale4(o[0], fzw), ez1 = scale4(o[1], fzw);
                /* x+1 neighbour: H_new(z-1) of the quad to the right */
                const float xp1 = fxp * lds4(&HS(ze, ry, 1) + xqn).x, xp2 = fxp * lds4(&HS(ze, ry, 2) + xqn).x;
                te.az = zi.ae;
                te.gz = zi.ge;
                const bool qae = qse || (REC && (isnan(ce[0].x) | isnan(ce[0].y) | isnan(ce[0].z) | isnan(ce[0].w)));
                row_quad<true, REC>(p, k, b, gy, ze, x0, ze == iIb, te, ce, Ep, hp, ae, ey0, ey2, ez0, ez1, xp1, xp2, pyze);
#pragma unroll
                for (int i = 0; i < 3; i++) st4(r.En + i * n3 + le, Ep[i]);
                if (qae) {
#pragma unroll
                    for (int i = 0; i < 3; i++) st4(r.Ean + i * n3 + le, ae[i]);
                }
                const int q = zi.q;
                if (q >= 0) {
                    st4(row_ring(p.d, g.pl, b, k, q, 2) + px0, Ep[0]);
                    st4(row_ring(p.d, g.pl, b, k, q, 3) + px0, Ep[1]);
                }
            }
            /* the private slot is free: plane z's be, E aux leave (G3) */
            if (own && z < z1) stage_e(z);
            cpa_commit();
            if (act) {
#pragma unroll
                for (int i = 0; i < 3; i++) Ep[i] = e[i];
            }
            /* the next plane's E (G1) complete, then visible to the neighbours */
            cpa_wait2();
            __syncthreads();
        }
    }
#undef ES
#undef PH
#undef PE
#undef TOP
#undef HS
}

/* The metal cells of a step of form 6, after it: the stable-form E update,
 * whose backward curls read H_new of the plane below and of the row above
 * the cell (values the march no longer holds, or another CTA's), and the
 * monitor samples of stable-form and frozen components, which are the main
 * slot rather than the total field -- the sweeps' general-cell path
 * (fdtd_f32.cu, general32_cell) on the old set (E, H aux, E aux) and the new
 * one (H, H aux).  One thread per cell and excitation (blockIdx.y): the nh
 * H cells, then the ne E cells. */
__global__ void __launch_bounds__(128) k_row_metal(const Row32 r, const int rel, const int *hcells, const int nh,
                                                   const int *ecells, const int ne)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nh + ne) return;
    const P32 &p = r.p;
    const Geo &g = p.g;
    const int b = blockIdx.y;
    const bool ef = i >= nh;
    const long long l = ef ? ecells[i - nh] : hcells[i];
    const long long n3 = g.n3, bs = 3 * n3;
    const int j0 = (int)(l % g.L0), j1 = (int)((l / g.L0) % g.L1), j2 = (int)(l / g.pl);
    const int q = row_monitor(p.d, j2);
    const Rec32 rc = (ef ? p.erec : p.hrec)[__float_as_int((ef ? p.be : p.bh)[n3 + l])];
    if (q < 0 && !(ef && rc.kind == RK_STABLE)) return; /* nothing else to do off the monitor planes */
    const float sg = ef ? 1.0f : -1.0f;
    const float *F = (ef ? p.E : p.H) + b * bs, *Fa = (ef ? p.Ea : p.Ha) + b * bs; /* the old set */
    float mo[3];
    if (rc.kind == RK_FROZEN) {
        for (int c = 0; c < 3; c++) mo[c] = F[c * n3 + l] - Fa[c * n3 + l];
    } else {
        /* the stable form differentiates the MAIN slot of the other field */
        const float *G = ef ? r.Hn + b * bs : p.E + b * bs, *Ga = ef ? r.Han + b * bs : p.Ea + b * bs;
        const Stn32 st = make_stn32(g, j0, j1, j2, false);
        auto get = [&](int c, long long o) { return G[c * n3 + l + o] - Ga[c * n3 + l + o]; };
        float pl[3], mi[3];
        curl32<false>(get, st, pl, mi);
        for (int c = 0; c < 3; c++) {
            const float W = pl[c] + mi[c];
            float x = Fa[c * n3 + l];
            float f = F[c * n3 + l] - x;
            f += 0.5f * x;
            x = fmaf(sg * rc.B1[c], W, rc.A1[c] * x);
            f += 0.5f * x;
            mo[c] = f;
            if (ef) {
                r.En[b * bs + c * n3 + l] = f + x;
                r.Ean[b * bs + c * n3 + l] = x;
            }
        }
    }
    if (q >= 0) {
        const int k = *p.s.base + rel;
        const int px = j0 + g.L0 * j1;
        row_ring(p.d, g.pl, b, k, q, ef ? 2 : 0)[px] = mo[0];
        row_ring(p.d, g.pl, b, k, q, ef ? 3 : 1)[px] = mo[1];
    }
}

template <int MAXT, int MB, bool REC>
__global__ void __launch_bounds__(MAXT, MB) k_row32(const Row32 r, const int rel)
{
    /* CTAs in order of excitation fastest (the coefficient stream is shared
     * by the CTAs of one row tile and plane range), then item group; the
     * pieces (row tile, planes [z0, z1)) of excitation b this CTA marches */
    const int b = blockIdx.x % r.p.batch, gidx = blockIdx.x / r.p.batch;
    RowPieces work(r.nyt, r.p.g.L2, r.zc, r.ngroups, gidx);
    row_march<REC>(r, rel, b, [&](int &yt, int &z0, int &z1) { return work.next(r.nyt, r.p.g.L2, r.zc, gidx, yt, z0, z1); });
}

/* A group of plans in one persistent launch: CTA blockIdx.x belongs to the
 * member whose CTA range holds it and runs that member's own persistent
 * schedule there (a group of one CTA per excitation marching the same pieces,
 * so that the excitations of a tile share the coefficient stream through L2).
 * The member's parameters are read in place from the parameter space at an
 * offset that is uniform over the CTA (derived from blockIdx only), so they
 * stay in uniform registers: a copy in shared memory, or an index loaded from
 * memory, cost a quarter of the step's speed. */
template <int MAXT, int MB, bool REC>
__global__ void __launch_bounds__(MAXT, MB) k_row32g(const __grid_constant__ RowGroup32 G, const int rel)
{
    int m = 0;
    while (m + 1 < G.n && (int)blockIdx.x >= G.first[m + 1]) m++;
    const Row32 &r = G.r[m];
    const int c = (int)blockIdx.x - G.first[m];
    const int b = c % r.p.batch, gidx = c / r.p.batch;
    RowPieces work(r.nyt, r.p.g.L2, 0, r.ngroups, gidx);
    row_march<REC>(r, rel, b, [&](int &yt, int &z0, int &z1) { return work.next(r.nyt, r.p.g.L2, 0, gidx, yt, z0, z1); });
}

template <int MAXT, int MB, bool REC> const void *row_fn() { return (const void *)k_row32<MAXT, MB, REC>; }

/* the grouped launch: 384 threads at one CTA per SM or 192 at two (the
 * register bound of the single-plan instantiations of those shapes) */
const void *row_group_kernel(int threads, bool rec)
{
    if (threads == 384) return rec ? (const void *)k_row32g<384, 1, true> : (const void *)k_row32g<384, 1, false>;
    if (threads == 192) return rec ? (const void *)k_row32g<192, 2, true> : (const void *)k_row32g<192, 2, false>;
    return nullptr;
}

/* the instantiation for a block of `threads` at register bound mb (at least
 * mb resident CTAs of MAXT threads: 65536 / (MAXT * mb) registers), or null;
 * plans with record cells: one CTA per SM only */
const void *row_kernel(int threads, int mb, bool rec)
{
    if (rec) {
        if (mb != 1) return nullptr;
        if (threads <= 384) return row_fn<384, 1, true>();
        if (threads <= 640) return row_fn<640, 1, true>();
        if (threads <= 1024) return row_fn<1024, 1, true>();
        return nullptr;
    }
    switch (mb) {
    case 1:
        if (threads <= 384) return row_fn<384, 1, false>();
        if (threads <= 448) return row_fn<448, 1, false>();
        if (threads <= 512) return row_fn<512, 1, false>();
        if (threads <= 640) return row_fn<640, 1, false>();
        if (threads <= 1024) return row_fn<1024, 1, false>();
        return nullptr;
    case 2:
        if (threads <= 192) return row_fn<192, 2, false>();
        if (threads <= 384) return row_fn<384, 2, false>();
        return nullptr;
    case 3: return threads <= 256 ? row_fn<256, 3, false>() : nullptr;
    default: return nullptr;
    }
}

} // namespace

int row32_threads(int L0, int ty) { return ((L0 / 4 * (ty + 1) + 31) / 32) * 32; }

} // namespace smat

/* The pieces CTA group gidx of launch form 6 marches (the kernel's own
 * schedule, run on the host): {row tile, z0, z1} triples into out (room for
 * max_pieces), their count in *n.  For checking that the pieces of all groups
 * partition the grid. */
extern "C" int smat_row32_pieces(int L1, int L2, int tile_y, int z_chunk, int ngroups, int gidx, int *out,
                                 int max_pieces, int *n)
{
    if (L1 < 1 || L2 < 1 || tile_y < 1 || z_chunk < 0 || ngroups < 0 || gidx < 0 || !out || !n || max_pieces < 0)
        return smat_fail(SMAT_EINVAL, "row32_pieces: bad arguments");
    const int nyt = (L1 + tile_y - 1) / tile_y;
    const int zc = z_chunk >= L2 ? L2 : z_chunk;
    if (zc > 0 && gidx >= nyt * ((L2 + zc - 1) / zc))
        return smat_fail(SMAT_EINVAL, "row32_pieces: item %d beyond the %d chunked items", gidx,
                         nyt * ((L2 + zc - 1) / zc));
    if (zc == 0 && gidx >= (ngroups > 0 ? ngroups : 1))
        return smat_fail(SMAT_EINVAL, "row32_pieces: group %d beyond the %d groups", gidx, ngroups);
    smat::RowPieces w(nyt, L2, zc, ngroups, gidx);
    int yt, z0, z1, k = 0;
    while (w.next(nyt, L2, zc, gidx, yt, z0, z1)) {
        if (k >= max_pieces) return smat_fail(SMAT_EINVAL, "row32_pieces: more than %d pieces", max_pieces);
        out[3 * k] = yt;
        out[3 * k + 1] = z0;
        out[3 * k + 2] = z1;
        k++;
    }
    *n = k;
    return SMAT_OK;
}

namespace smat {

size_t row32_smem(int L0, int ty, int zc) { return sizeof(float4) * row_smem_f4(L0, ty, zc); }

/* Lets fn take up to the device's opt-in maximum of dynamic shared memory.
 * One limit for every launch of a kernel: several plans (a group's members)
 * share one instantiation with different staging sizes, so a limit lowered
 * for one plan must not refuse another's launch. */
bool allow_max_smem(const void *fn, size_t need)
{
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, fn) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const long long room = (long long)optin - (long long)fa.sharedSizeBytes;
    if (room < (long long)need) return false;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)room) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return true;
}

int row32_max_ctas_per_sm(int L0, int ty, int mb, int zc, bool rec)
{
    const int threads = row32_threads(L0, ty);
    const void *fn = row_kernel(threads, mb, rec);
    if (!fn) return 0;
    const size_t sm = row32_smem(L0, ty, zc);
    if (!allow_max_smem(fn, sm)) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, sm) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int row32_group_max_ctas_per_sm(int threads, size_t smem, bool rec)
{
    const void *fn = row_group_kernel(threads, rec);
    if (!fn) return 0;
    if (!allow_max_smem(fn, smem)) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

void launch_row32_group(const RowGroup32 &g, int rel, int threads, int grid, size_t smem, bool rec, cudaStream_t st)
{
    void *args[] = {(void *)&g, (void *)&rel};
    cudaLaunchKernel(row_group_kernel(threads, rec), dim3(grid), dim3(threads), args, smem, st);
}

void launch_row_metal(const Row32 &r, int rel, const int *hcells, int nh, const int *ecells, int ne, cudaStream_t st)
{
    if (nh + ne <= 0) return;
    k_row_metal<<<dim3((nh + ne + 127) / 128, r.p.batch), 128, 0, st>>>(r, rel, hcells, nh, ecells, ne);
}

void launch_row32(const Row32 &r, int rel, int mb, cudaStream_t st)
{
    const int nt = row32_threads(r.p.g.L0, r.ty);
    const dim3 blk(nt);
    const void *fn = row_kernel(nt, mb, r.has_rec != 0);
    const size_t sm = row32_smem(r.p.g.L0, r.ty, r.zc > 0 ? r.zc : r.p.g.L2);
    void *args[] = {(void *)&r, (void *)&rel};
    cudaLaunchKernel(fn, dim3(r.nitems), blk, args, sm, st);
}

} // namespace smat
