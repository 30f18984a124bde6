/*
 * FP32 split-field FDTD: one fused, persistent launch per Yee step.
 *
 * Same update as the two FP32 sweeps in fdtd_f32.cu (and the same floating
 * point expressions, so results are bit-identical to them), reorganised for
 * HBM bandwidth:
 *
 *   - a CTA owns an (x, y) tile of 32 x TY cells of one excitation and marches
 *     along z through a chunk of planes.  At plane z it computes H_new(z) on
 *     the tile plus a +1 halo column and row, then E_new(z-1) on the tile: the
 *     E update one plane behind consumes H_new of planes z-1 and z from shared
 *     memory, so each step reads E, H and the coefficients once and writes E
 *     and H once (72 B per cell per excitation instead of the 96 B of two
 *     sweeps);
 *   - fields are double-buffered (read the "old" set, write the "new" set), so
 *     a CTA reading its neighbours' halo never sees a value another CTA has
 *     already advanced;
 *   - E planes (tile + 1-cell halo, 3 components) are staged in shared memory
 *     with cp.async four planes deep, and the per-cell data of the next plane
 *     (H, coefficients, aux slots) is prefetched into registers, so every
 *     thread keeps a plane of loads in flight while it computes;
 *   - work items (excitation fastest, then tile, then z chunk) are strided
 *     over a grid sized to the resident CTA count: one persistent launch, and
 *     the CTAs of the same tile for different excitations run together so the
 *     shared coefficient stream is read from HBM once;
 *   - halo positions that wrap around the domain hold iBc * value, the
 *     reference's boundary factor (FDTDsplitfieldMetal.c:334, :355): a wrapped
 *     halo H cell is computed from sign-flipped inputs, which for iBc = +-1 is
 *     exactly iBc * H_new of the wrapped cell (and set to 0 for iBc = 0);
 *   - stable-form ('e','b') E cells need H_new of backward neighbours that may
 *     belong to another tile; they are finished by a small fix-up kernel after
 *     the fused launch (k_fix_stable32).
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"

namespace smat {

constexpr int TX = 32;
constexpr int SEX = TX + 2; /* row stride of the staged E planes */
constexpr int SHX = TX + 1; /* row stride of the H_new planes */
constexpr int NSH = 3;      /* H_new planes kept */
constexpr int EPOS = 3;     /* E staging positions per thread: (32+2)(TY+2) <= 3*32*TY for TY >= 2 */

__device__ __forceinline__ void cp_async4(float *smem, const float *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ int wrapc(int v, int n, int bc, float &f)
{
    if (v < 0) {
        f *= (float)bc;
        return v + n;
    }
    if (v >= n) {
        f *= (float)bc;
        return v - n;
    }
    return v;
}

__device__ __forceinline__ double sheet_f(const Src &s, int pl, int b, int k, bool efield, int v, int p)
{
    if (s.xsrc) return s.xsrc[(efield ? 2 * pl : 0) + v + 2 * p];
    const double *sc = s.sched + 6 * (long long)k + (efield ? 0 : 3);
    const double *w = s.inc + (long long)b * 8 * pl + (efield ? 4 * pl : 0) + 2 * (v + 2 * p);
    return sc[0] * (sc[1] * w[0] + sc[2] * w[1]);
}

__device__ __forceinline__ int mon_index(const Dft &d, int z)
{
    int q = -1;
#pragma unroll
    for (int i = 0; i < MAX_PLANES; i++)
        if (i < d.nq && d.planes[i] == z) q = i;
    return q;
}

__device__ __forceinline__ float *ring_ptr(const Dft &d, int pl, int b, int k, int q, int v)
{
    const int slot = k % d.ringK;
    return d.ring + ((((long long)b * d.ringK + slot) * d.nq + q) * 4 + v) * (long long)pl;
}

/* ---- the general (record) path, global memory, old buffers -------------- */

/* H_new (total), aux and main of one cell from its record; (gx,gy,gz) actual
 * cell.  Out of line: general cells are rare and must not cost the hot path
 * registers. */
__device__ __noinline__ void h_general(const Fused32 &f, int b, int k, int gx, int gy, int gz, int ridx,
                                       float *out_T, float *out_m, float *out_main)
{
    const P32 &p = f.p;
    const Geo &g = p.g;
    const Rec32 r = p.hrec[ridx];
    const long long n3 = g.n3, bs = 3 * n3;
    const long long l = gx + (long long)g.L0 * (gy + (long long)g.L1 * gz);
    const float *T = p.H + b * bs, *M = p.Ha + b * bs, *E = p.E + b * bs, *Ea = p.Ea + b * bs;
    float t[3], m[3];
    for (int c = 0; c < 3; c++) {
        t[c] = T[c * n3 + l];
        m[c] = M[c * n3 + l];
    }
    if (r.kind == RK_FROZEN) {
        for (int c = 0; c < 3; c++) {
            out_T[c] = t[c];
            out_m[c] = m[c];
            out_main[c] = t[c] - m[c];
        }
        return;
    }
    /* backward neighbours with boundary factors */
    const int j[3] = {gx, gy, gz};
    const int L[3] = {g.L0, g.L1, g.L2};
    long long off[3];
    float fb[3];
    long long stride = 1;
    for (int a = 0; a < 3; a++) {
        const bool edge = j[a] == 0;
        off[a] = (long long)((edge ? L[a] - 1 : j[a] - 1) - j[a]) * stride;
        fb[a] = edge ? (float)g.bc[a] : 1.0f;
        stride *= L[a];
    }
    const bool stable = r.kind == RK_STABLE;
    auto get = [&](int c, int a) -> float { /* a = -1: here */
        const long long i = c * n3 + l + (a < 0 ? 0 : off[a]);
        const float v = stable ? E[i] - Ea[i] : E[i];
        return a < 0 ? v : fb[a] * v;
    };
    float pl[3], mi[3];
    for (int c = 0; c < 3; c++) {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        pl[c] = get(a2, -1) - get(a2, a1);
        mi[c] = get(a1, a2) - get(a1, -1);
    }
    if (stable) {
        for (int c = 0; c < 3; c++) {
            const float W = pl[c] + mi[c];
            float x = m[c];
            float fm = t[c] - x;
            fm += 0.5f * x;
            x = fmaf(-1.0f * r.B1[c], W, r.A1[c] * x);
            fm += 0.5f * x;
            out_main[c] = fm;
            out_T[c] = fm + x;
            out_m[c] = x;
        }
    } else if (r.kind == RK_N) {
        float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
        if (gz == p.s.iI[b]) {
            const int px = gx + g.L0 * gy;
            W[0] += (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, true, 1, px));
            W[1] -= (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, true, 0, px));
        }
        for (int c = 0; c < 3; c++) {
            out_T[c] = fmaf(-1.0f * r.B0[c], W[c], r.A0[c] * t[c]);
            out_m[c] = m[c];
            out_main[c] = out_T[c];
        }
    } else { /* RK_A */
        for (int c = 0; c < 3; c++) {
            const float pp = t[c] - m[c];
            const float np = fmaf(-1.0f * r.B0[c], pl[c], r.A0[c] * pp);
            const float nm = fmaf(-1.0f * r.B1[c], mi[c], r.A1[c] * m[c]);
            out_T[c] = np + nm;
            out_m[c] = nm;
            out_main[c] = np + nm;
        }
    }
}

/* E_new of a general (record) cell other than the stable form; returns
 * whether the aux slot is written and the DFT sample (main) value. */
__device__ __noinline__ void e_general(const Fused32 &f, int b, int k, int gx, int gy, int zp, int ridx,
                                       const float *pl, const float *mi, const float *e0, float *eo, float *eom,
                                       float *emain)
{
    const P32 &p = f.p;
    const Geo &g = p.g;
    const Rec32 r = p.erec[ridx];
    const long long n3 = g.n3, bs = 3 * n3;
    const long long gi = gx + (long long)g.L0 * (gy + (long long)g.L1 * zp);
    const float *Eao = p.Ea + b * bs;
    if (r.kind == RK_FROZEN) {
        for (int c = 0; c < 3; c++) {
            eom[c] = Eao[c * n3 + gi];
            eo[c] = e0[c];
            emain[c] = e0[c] - eom[c];
        }
    } else if (r.kind == RK_N) {
        float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
        if (zp == p.s.iI[b]) {
            const int px = gx + g.L0 * gy;
            W[0] += (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, false, 1, px));
            W[1] -= (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, false, 0, px));
        }
        for (int c = 0; c < 3; c++) {
            eo[c] = fmaf(1.0f * r.B0[c], W[c], r.A0[c] * e0[c]);
            eom[c] = Eao[c * n3 + gi];
            emain[c] = eo[c];
        }
    } else { /* RK_A */
        for (int c = 0; c < 3; c++) {
            const float m = Eao[c * n3 + gi];
            const float pp = e0[c] - m;
            const float np = fmaf(1.0f * r.B0[c], pl[c], r.A0[c] * pp);
            const float nm = fmaf(1.0f * r.B1[c], mi[c], r.A1[c] * m);
            eo[c] = np + nm;
            eom[c] = nm;
            emain[c] = np + nm;
        }
    }
}

/* ---- the fused kernel ----------------------------------------------------- */

/* Shared memory per CTA, TY tile rows: NSE plane slots, each holding
 *   E     [3][TY+2][TX+2]  old E, tile + 1-cell halo (iBc-scaled where wrapped)
 *   Q     [3][3][TY+1][TX+1] old H (total), H coefficient, H aux: tile + the +1
 *                          halo column and row (iBc-scaled where wrapped)
 *   B     [2][3][TY][TX]   E coefficient, E aux: tile
 * and NSH planes of H_new [3][TY+1][TX+1]. */
__host__ __device__ constexpr int slot_floats(int ty)
{
    return 3 * (ty + 2) * SEX + 9 * (ty + 1) * SHX + 6 * ty * TX;
}

/* NS plane slots; planes are staged NS - 3 ahead of the one being computed
 * (a slot is free again three planes after it was staged). */
template <int NS>
__global__ void __launch_bounds__(256) k_fused32(const Fused32 f, const int rel)
{
    constexpr int DEPTH = NS - 3;
    extern __shared__ float smem[];
    const P32 &p = f.p;
    const Geo &g = p.g;
    const int TY = blockDim.y;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx, nthr = TX * TY;
    const int SEY = TY + 2, SHY = TY + 1;
    const int SLOT = slot_floats(TY);
    const int OQ = 3 * SEY * SEX, OB = OQ + 9 * SHY * SHX;
    float *sH = smem + NS * SLOT;
    const long long n3 = g.n3, bs = 3 * n3;
    const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
    const int S = L0 + L1 + L2, s1 = L0, s2 = L0 + L1;
    const long long pl = g.pl;
    const int k = *p.s.base + rel;
#define SE(s, c, ly, lx) smem[(s) * SLOT + ((c) * SEY + (ly)) * SEX + (lx)]
#define SQ(s, a, c, ly, lx) smem[(s) * SLOT + OQ + (((a) * 3 + (c)) * SHY + (ly)) * SHX + (lx)]
#define SB(s, a, c) smem[(s) * SLOT + OB + (((a) * 3 + (c)) * TY + ty) * TX + tx]
#define HN(s, c, ly, lx) sH[(((s) * 3 + (c)) * SHY + (ly)) * SHX + (lx)]

    for (int item = blockIdx.x; item < f.nitems; item += gridDim.x) {
        const int b = item % p.batch;
        int t = item / p.batch;
        const int tix = t % f.ntx;
        t /= f.ntx;
        const int tiy = t % f.nty;
        const int zci = t / f.nty;
        const int X0 = tix * TX, Y0 = tiy * TY;
        const int w = min(TX, L0 - X0), h = min(TY, L1 - Y0);
        const int z0 = zci * f.zc, z1 = min(z0 + f.zc, L2);
        const float *Eo = p.E + b * bs, *Ho = p.H + b * bs, *Hao = p.Ha + b * bs, *Eao = p.Ea + b * bs;
        float *En = f.En + b * bs, *Hn = f.Hn + b * bs, *Han = f.Han + b * bs, *Ean = f.Ean + b * bs;
        const bool own = tx < w && ty < h;
        const int gx = X0 + tx, gy = Y0 + ty;
        const int own2d = gx + L0 * gy;
        const bool own_split2d = own && (p.pmask[gx] | p.pmask[s1 + gy]);

        /* this thread's staging positions for the item (fixed over z) */
        const int nex = w + 2, npe = nex * (h + 2);
        int eoff[EPOS], elx[EPOS], ely[EPOS];
        float efac[EPOS];
#pragma unroll
        for (int q = 0; q < EPOS; q++) {
            const int i = tid + q * nthr;
            efac[q] = 0.0f;
            eoff[q] = -1;
            elx[q] = ely[q] = 0;
            if (i < npe) {
                elx[q] = i % nex;
                ely[q] = i / nex;
                float fc = 1.0f;
                const int xx = wrapc(X0 - 1 + elx[q], L0, g.bc[0], fc);
                const int yy = wrapc(Y0 - 1 + ely[q], L1, g.bc[1], fc);
                eoff[q] = xx + L0 * yy;
                efac[q] = fc;
            }
        }
        /* halo duty: the +1 column (lx = w) and row (ly = h) of H_new */
        int hlx = -1, hly = -1, hoff = 0, hxx = 0, hyy = 0;
        float hfac = 0.0f;
        bool hsplit2d = false;
        if (tid < h) {
            hlx = w;
            hly = tid;
        } else if (tid < h + w) {
            hlx = tid - h;
            hly = h;
        }
        if (hlx >= 0) {
            float fc = 1.0f;
            hxx = wrapc(X0 + hlx, L0, g.bc[0], fc);
            hyy = wrapc(Y0 + hly, L1, g.bc[1], fc);
            hoff = hxx + L0 * hyy;
            hfac = fc;
            hsplit2d = p.pmask[hxx] | p.pmask[s1 + hyy];
        }

        /* stage plane zl (logical: z0-1 .. z1) into slot (zl + NS) % NS */
        auto stage = [&](int zl) {
            const int sl = (zl + NS) % NS;
            float fz = 1.0f;
            const int gz = wrapc(zl, L2, g.bc[2], fz);
            const long long base = pl * gz;
#pragma unroll
            for (int q = 0; q < EPOS; q++) {
                if (eoff[q] < 0) continue;
                const float fc = efac[q] * fz;
                const long long gi = base + eoff[q];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    float *d = &SE(sl, c, ely[q], elx[q]);
                    if (fc == 1.0f) cp_async4(d, Eo + c * n3 + gi);
                    else *d = fc * Eo[c * n3 + gi];
                }
            }
            if (zl < z0) return; /* the pre-plane only feeds the z-derivative */
            const bool zsplit = p.pmask[s2 + gz];
            if (own) {
                const long long gi = base + own2d;
                const bool split = own_split2d | zsplit;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    float *dT = &SQ(sl, 0, c, ty, tx);
                    if (fz == 1.0f) cp_async4(dT, Ho + c * n3 + gi);
                    else *dT = fz * Ho[c * n3 + gi];
                    cp_async4(&SQ(sl, 1, c, ty, tx), p.bh + c * n3 + gi);
                    if (split) {
                        float *dm = &SQ(sl, 2, c, ty, tx);
                        if (fz == 1.0f) cp_async4(dm, Hao + c * n3 + gi);
                        else *dm = fz * Hao[c * n3 + gi];
                    }
                }
                if (zl < z1) {
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        cp_async4(&SB(sl, 0, c), p.be + c * n3 + gi);
                        if (split) cp_async4(&SB(sl, 1, c), Eao + c * n3 + gi);
                    }
                }
            }
            if (hlx >= 0 && zl < z1) {
                const long long gi = base + hoff;
                const float fc = hfac * fz;
                const bool split = hsplit2d | zsplit;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    float *dT = &SQ(sl, 0, c, hly, hlx);
                    if (fc == 1.0f) cp_async4(dT, Ho + c * n3 + gi);
                    else *dT = fc * Ho[c * n3 + gi];
                    cp_async4(&SQ(sl, 1, c, hly, hlx), p.bh + c * n3 + gi);
                    if (split) {
                        float *dm = &SQ(sl, 2, c, hly, hlx);
                        if (fc == 1.0f) cp_async4(dm, Hao + c * n3 + gi);
                        else *dm = fc * Hao[c * n3 + gi];
                    }
                }
            }
        };

        /* H_new of plane z at tile position (lx, ly) */
        auto h_update = [&](int z, int lx, int ly, int xx, int yy, float fxy, bool split2d, float o[3], float om[3],
                            float omain[3], bool &wa) {
            wa = false;
            const int sc = (z + NS) % NS, sp = (z + NS - 1) % NS;
            float fac = fxy;
            const int gz = wrapc(z, L2, g.bc[2], fac);
            if (fac == 0.0f) { /* wrapped with iBc = 0: iBc * H_new = 0 */
#pragma unroll
                for (int c = 0; c < 3; c++) o[c] = om[c] = omain[c] = 0.0f;
                return;
            }
            const float c0 = SQ(sc, 1, 0, ly, lx);
            if (isnan(c0)) {
                /* out-of-line results go through a local buffer touched only here,
                 * so the hot path's values stay in registers */
                float tmp[9];
                h_general(f, b, k, xx, yy, gz, __float_as_int(SQ(sc, 1, 1, ly, lx)), tmp, tmp + 3, tmp + 6);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    o[c] = tmp[c] * fac;
                    om[c] = tmp[3 + c] * fac;
                    omain[c] = tmp[6 + c] * fac;
                }
                wa = true;
                return;
            }
            const int ex = lx + 1, ey = ly + 1;
            const float Ex = SE(sc, 0, ey, ex), Ey = SE(sc, 1, ey, ex), Ez = SE(sc, 2, ey, ex);
            const float pl_[3] = {Ez - SE(sc, 2, ey - 1, ex), Ex - SE(sp, 0, ey, ex), Ey - SE(sc, 1, ey, ex - 1)};
            const float mi_[3] = {SE(sp, 1, ey, ex) - Ey, SE(sc, 2, ey, ex - 1) - Ez, SE(sc, 0, ey - 1, ex) - Ex};
            const bool split = split2d | p.pmask[s2 + gz];
            if (!split) {
                float W[3] = {pl_[0] + mi_[0], pl_[1] + mi_[1], pl_[2] + mi_[2]};
                if (gz == p.s.iI[b]) {
                    const int px = xx + L0 * yy;
                    W[0] += fac * (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, true, 1, px));
                    W[1] -= fac * (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, true, 0, px));
                }
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    o[c] = fmaf(-1.0f * SQ(sc, 1, c, ly, lx), W[c], SQ(sc, 0, c, ly, lx));
                    om[c] = 0.0f;
                    omain[c] = o[c];
                }
            } else {
                const int jx[3] = {xx, s1 + yy, s2 + gz};
                const float *tA = p.tab, *tG = p.tab + S;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const int i1 = jx[(c + 1) % 3], i2 = jx[(c + 2) % 3];
                    const float bn = SQ(sc, 1, c, ly, lx);
                    const float Ap = tA[i1], Bp = -1.0f * bn * tG[i1];
                    const float Am = tA[i2], Bm = -1.0f * bn * tG[i2];
                    const float m = SQ(sc, 2, c, ly, lx);
                    const float pp = SQ(sc, 0, c, ly, lx) - m;
                    const float np = fmaf(Bp, pl_[c], Ap * pp);
                    const float nm = fmaf(Bm, mi_[c], Am * m);
                    o[c] = np + nm;
                    om[c] = nm;
                    omain[c] = np + nm;
                }
                wa = true;
            }
        };

        stage(z0 - 1);
        cp_async_commit();
#pragma unroll
        for (int d = 0; d < DEPTH; d++) {
            if (z0 + d <= z1) stage(z0 + d);
            cp_async_commit();
        }
        for (int z = z0; z <= z1; z++) {
            if (z + DEPTH <= z1) stage(z + DEPTH);
            cp_async_commit();
            cp_async_wait<DEPTH>();
            __syncthreads();

            /* ---- H_new(z): own cell and halo duty -> H_new plane ---- */
            const int hs = (z - z0) % NSH;
            if (own) {
                float o[3], om[3], omain[3];
                bool wa;
                h_update(z, tx, ty, gx, gy, 1.0f, own_split2d, o, om, omain, wa);
#pragma unroll
                for (int c = 0; c < 3; c++) HN(hs, c, ty, tx) = o[c];
                if (z < z1) {
                    const long long gi = own2d + pl * z;
#pragma unroll
                    for (int c = 0; c < 3; c++) Hn[c * n3 + gi] = o[c];
                    if (wa) {
#pragma unroll
                        for (int c = 0; c < 3; c++) Han[c * n3 + gi] = om[c];
                    }
                    const int q = mon_index(p.d, z);
                    if (q >= 0) {
                        ring_ptr(p.d, g.pl, b, k, q, 0)[own2d] = omain[0];
                        ring_ptr(p.d, g.pl, b, k, q, 1)[own2d] = omain[1];
                    }
                }
            }
            if (hlx >= 0 && z < z1) {
                float o[3], om[3], omain[3];
                bool wa;
                h_update(z, hlx, hly, hxx, hyy, hfac, hsplit2d, o, om, omain, wa);
#pragma unroll
                for (int c = 0; c < 3; c++) HN(hs, c, hly, hlx) = o[c];
            }
            __syncthreads();

            /* ---- E_new(z-1) on the tile ---- */
            if (z > z0 && own) {
                const int zp = z - 1;
                const int hp = (zp - z0) % NSH;
                const int se = (zp + NS) % NS;
                const float Hx = HN(hp, 0, ty, tx), Hy = HN(hp, 1, ty, tx), Hz = HN(hp, 2, ty, tx);
                const float pl_[3] = {HN(hp, 2, ty + 1, tx) - Hz, HN(hs, 0, ty, tx) - Hx, HN(hp, 1, ty, tx + 1) - Hy};
                const float mi_[3] = {Hy - HN(hs, 1, ty, tx), Hz - HN(hp, 2, ty, tx + 1), Hx - HN(hp, 0, ty + 1, tx)};
                const float e0[3] = {SE(se, 0, ty + 1, tx + 1), SE(se, 1, ty + 1, tx + 1), SE(se, 2, ty + 1, tx + 1)};
                const long long gi = own2d + pl * zp;
                const float c0 = SB(se, 0, 0);
                float eo[3], eom[3], emain[3];
                bool done = true, wa = false;
                if (!isnan(c0)) {
                    const bool split = own_split2d | p.pmask[s2 + zp];
                    if (!split) {
                        float W[3] = {pl_[0] + mi_[0], pl_[1] + mi_[1], pl_[2] + mi_[2]};
                        if (zp == p.s.iI[b]) {
                            W[0] += (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, false, 1, own2d));
                            W[1] -= (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, false, 0, own2d));
                        }
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            eo[c] = fmaf(1.0f * SB(se, 0, c), W[c], e0[c]);
                            emain[c] = eo[c];
                        }
                    } else {
                        const int jx[3] = {gx, s1 + gy, s2 + zp};
                        const float *tA = p.tab + 2 * S, *tG = p.tab + 3 * S;
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            const int i1 = jx[(c + 1) % 3], i2 = jx[(c + 2) % 3];
                            const float bn = SB(se, 0, c);
                            const float Ap = tA[i1], Bp = 1.0f * bn * tG[i1];
                            const float Am = tA[i2], Bm = 1.0f * bn * tG[i2];
                            const float m = SB(se, 1, c);
                            const float pp = e0[c] - m;
                            const float np = fmaf(Bp, pl_[c], Ap * pp);
                            const float nm = fmaf(Bm, mi_[c], Am * m);
                            eo[c] = np + nm;
                            eom[c] = nm;
                            emain[c] = np + nm;
                        }
                        wa = true;
                    }
                } else {
                    const int ridx = __float_as_int(SB(se, 0, 1));
                    if (p.erec[ridx].kind == RK_STABLE) {
                        done = false; /* finished by k_fix_stable32 */
                    } else {
                        float tmp[18];
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            tmp[c] = pl_[c];
                            tmp[3 + c] = mi_[c];
                            tmp[6 + c] = e0[c];
                        }
                        e_general(f, b, k, gx, gy, zp, ridx, tmp, tmp + 3, tmp + 6, tmp + 9, tmp + 12, tmp + 15);
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            eo[c] = tmp[9 + c];
                            eom[c] = tmp[12 + c];
                            emain[c] = tmp[15 + c];
                        }
                        wa = true;
                    }
                }
                if (done) {
#pragma unroll
                    for (int c = 0; c < 3; c++) En[c * n3 + gi] = eo[c];
                    if (wa) {
#pragma unroll
                        for (int c = 0; c < 3; c++) Ean[c * n3 + gi] = eom[c];
                    }
                    const int q = mon_index(p.d, zp);
                    if (q >= 0) {
                        ring_ptr(p.d, g.pl, b, k, q, 2)[own2d] = emain[0];
                        ring_ptr(p.d, g.pl, b, k, q, 3)[own2d] = emain[1];
                    }
                }
            }
        }
        cp_async_wait0();
        __syncthreads();
    }
#undef SE
#undef SQ
#undef SB
#undef HN
}

/* stable-form E cells ('e', 'b'), after the fused launch: the reference's
 * backward difference of the H main slot (FDTDsplitfieldMetal.c:308-314) */
__global__ void k_fix_stable32(const Fused32 f, const int rel)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (i >= f.nstable) return;
    const P32 &p = f.p;
    const Geo &g = p.g;
    const long long n3 = g.n3, bs = 3 * n3;
    const long long l = f.stable[i];
    const int gx = (int)(l % g.L0), gy = (int)((l / g.L0) % g.L1), gz = (int)(l / ((long long)g.L0 * g.L1));
    const Rec32 r = p.erec[__float_as_int(p.be[n3 + l])];
    const float *Hn = f.Hn + b * bs, *Han = f.Han + b * bs, *Eo = p.E + b * bs, *Eao = p.Ea + b * bs;
    float *En = f.En + b * bs, *Ean = f.Ean + b * bs;
    const int j[3] = {gx, gy, gz};
    const int L[3] = {g.L0, g.L1, g.L2};
    long long off[3];
    float fb[3];
    long long stride = 1;
    for (int a = 0; a < 3; a++) {
        const bool edge = j[a] == 0;
        off[a] = (long long)((edge ? L[a] - 1 : j[a] - 1) - j[a]) * stride;
        fb[a] = edge ? (float)g.bc[a] : 1.0f;
        stride *= L[a];
    }
    auto get = [&](int c, int a) -> float {
        const long long ii = c * n3 + l + (a < 0 ? 0 : off[a]);
        const float v = Hn[ii] - Han[ii];
        return a < 0 ? v : fb[a] * v;
    };
    const int k = *p.s.base + rel;
    float mo[3];
    for (int c = 0; c < 3; c++) {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        const float W = (get(a2, -1) - get(a2, a1)) + (get(a1, a2) - get(a1, -1));
        float x = Eao[c * n3 + l];
        float fm = Eo[c * n3 + l] - x;
        fm += 0.5f * x;
        x = fmaf(1.0f * r.B1[c], W, r.A1[c] * x);
        fm += 0.5f * x;
        En[c * n3 + l] = fm + x;
        Ean[c * n3 + l] = x;
        mo[c] = fm;
    }
    const int q = mon_index(p.d, gz);
    if (q >= 0) {
        ring_ptr(p.d, g.pl, b, k, q, 2)[gx + g.L0 * gy] = mo[0];
        ring_ptr(p.d, g.pl, b, k, q, 3)[gx + g.L0 * gy] = mo[1];
    }
}

size_t fused32_smem(int ty, int ns)
{
    return sizeof(float) * ((size_t)ns * slot_floats(ty) + (size_t)NSH * 3 * (ty + 1) * SHX);
}

static void *fused_kernel(int ns)
{
    switch (ns) {
    case 4: return (void *)k_fused32<4>;
    case 5: return (void *)k_fused32<5>;
    default: return (void *)k_fused32<6>;
    }
}

int fused32_max_ctas_per_sm(int ty, int ns)
{
    int n = 0;
    const size_t sm = fused32_smem(ty, ns);
    cudaFuncSetAttribute(fused_kernel(ns), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fused_kernel(ns), TX * ty, sm) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

void launch_fused32(const Fused32 &f, int rel, int grid, cudaStream_t st)
{
    dim3 blk(TX, f.ty, 1);
    const size_t sm = fused32_smem(f.ty, f.ns);
    if (f.ns == 4) k_fused32<4><<<grid, blk, sm, st>>>(f, rel);
    else if (f.ns == 5) k_fused32<5><<<grid, blk, sm, st>>>(f, rel);
    else k_fused32<6><<<grid, blk, sm, st>>>(f, rel);
    if (f.nstable > 0) {
        dim3 g2((f.nstable + 127) / 128, f.p.batch);
        k_fix_stable32<<<g2, 128, 0, st>>>(f, rel);
    }
}


/* ===========================================================================
 * k_fused32t: the fused step with TMA plane staging (sm_90+ bulk tensor copies)
 *
 * Same computation and bit-identical results as k_fused32; the difference is
 * how a plane reaches shared memory: one elected thread issues a handful of
 * cp.async.bulk.tensor copies per plane (E tile + 1-cell halo, H / coefficient
 * / aux tiles with the +1 halo, E-side tiles) that complete on the slot's
 * mbarrier, instead of every thread issuing ~20 four-byte copies.  Needs
 * L0 % 4 == 0 (16-byte global strides).  Halo entries outside the domain come
 * back zero-filled; where the boundary factor iBc is +-1 they are patched with
 * iBc * (the wrapped value) after the copy lands, on boundary tiles only; a
 * plane wrapped along z is fetched at its wrapped index and scaled.
 * ========================================================================= */

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

/* bounded wait on the phase `parity` of bar; false on timeout */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    const unsigned a = smem_u32(bar);
    for (int it = 0; it < (1 << 24); it++) {
        unsigned done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load4(float *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                          uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4, %5}], [%6];\n" ::"r"(smem_u32(dst)),
                 "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
                 "r"(smem_u32(bar))
                 : "memory");
}

constexpr int TEX = TX + 8; /* E box width: x from X0-4 (16-byte aligned start) */
constexpr int TQX = TX + 4; /* H-side box width: x from X0 to X0+35 (covers the +1 halo) */

struct TSlot { /* float offsets inside one slot, each segment 128-byte aligned */
    int e, qt, qb, qm, be, bm, size;
};

__host__ __device__ inline int align32f(int n) { return (n + 31) & ~31; }

__host__ __device__ inline TSlot tslot(int ty)
{
    TSlot s;
    int o = 0;
    s.e = o;
    o += align32f(3 * (ty + 2) * TEX);
    s.qt = o;
    o += align32f(3 * (ty + 1) * TQX);
    s.qb = o;
    o += align32f(3 * (ty + 1) * TQX);
    s.qm = o;
    o += align32f(3 * (ty + 1) * TQX);
    s.be = o;
    o += align32f(3 * ty * TX);
    s.bm = o;
    o += align32f(3 * ty * TX);
    s.size = o;
    return s;
}

template <int NS>
__global__ void __launch_bounds__(256) k_fused32t(const __grid_constant__ Fused32T ft, const int rel)
{
    extern __shared__ __align__(128) float smem[];
    constexpr int DEPTH = NS - 3;
    const Fused32 &f = ft.f;
    const P32 &p = f.p;
    const Geo &g = p.g;
    const int TY = blockDim.y;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx, nthr = TX * TY;
    const TSlot sl = tslot(TY);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);       /* NS mbarriers (first 128 bytes) */
    float *slots = smem + 32;                                  /* NS slots */
    float *sH = slots + NS * sl.size;                          /* NSH planes of H_new */
    const int SHY = TY + 1;
    const long long n3 = g.n3, bs = 3 * n3;
    const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
    const int S = L0 + L1 + L2, s1 = L0, s2 = L0 + L1;
    const long long pl = g.pl;
    const int k = *p.s.base + rel;
#define TE(s, c, ly, lx) slots[(s) * sl.size + sl.e + ((c) * (TY + 2) + (ly)) * TEX + (lx)]
#define TQ(s, seg, c, ly, lx) slots[(s) * sl.size + (seg) + ((c) * (TY + 1) + (ly)) * TQX + (lx)]
#define TB(s, seg, c) slots[(s) * sl.size + (seg) + ((c) * TY + ty) * TX + tx]
#define HN(s, c, ly, lx) sH[(((s) * 3 + (c)) * SHY + (ly)) * SHX + (lx)]

    for (int item = blockIdx.x; item < f.nitems; item += gridDim.x) {
        const int b = item % p.batch;
        int t = item / p.batch;
        const int tix = t % f.ntx;
        t /= f.ntx;
        const int tiy = t % f.nty;
        const int zci = t / f.nty;
        const int X0 = tix * TX, Y0 = tiy * TY;
        const int w = min(TX, L0 - X0), h = min(TY, L1 - Y0);
        const int z0 = zci * f.zc, z1 = min(z0 + f.zc, L2);
        const float *Eo = p.E + b * bs, *Ho = p.H + b * bs, *Hao = p.Ha + b * bs;
        float *En = f.En + b * bs, *Hn = f.Hn + b * bs, *Han = f.Han + b * bs, *Ean = f.Ean + b * bs;
        const bool own = tx < w && ty < h;
        const int gx = X0 + tx, gy = Y0 + ty;
        const int own2d = gx + L0 * gy;
        const bool own_split2d = own && (p.pmask[gx] | p.pmask[s1 + gy]);
        const bool edge_tile = X0 == 0 || X0 + w == L0 || Y0 == 0 || Y0 + h == L1;
        /* does the tile (with its halo) hold any split cell in x or y? */
        bool tile_split2d = false;
        for (int x = X0 - 1; x <= X0 + w; x++) tile_split2d |= p.pmask[(x + L0) % L0] != 0;
        for (int y = Y0 - 1; y <= Y0 + h; y++) tile_split2d |= p.pmask[s1 + (y + L1) % L1] != 0;
        int hlx = -1, hly = -1, hxx = 0, hyy = 0;
        float hfac = 0.0f;
        bool hsplit2d = false;
        if (tid < h) {
            hlx = w;
            hly = tid;
        } else if (tid < h + w) {
            hlx = tid - h;
            hly = h;
        }
        if (hlx >= 0) {
            float fc = 1.0f;
            hxx = wrapc(X0 + hlx, L0, g.bc[0], fc);
            hyy = wrapc(Y0 + hly, L1, g.bc[1], fc);
            hfac = fc;
            hsplit2d = p.pmask[hxx] | p.pmask[s1 + hyy];
        }
        if (tid == 0)
            for (int s = 0; s < NS; s++) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        __syncthreads();

        /* producer (thread 0): all copies of logical plane zl into its slot */
        auto issue = [&](int zl) {
            const int s = (zl + NS) % NS;
            float fz = 1.0f;
            int gz = wrapc(zl, L2, g.bc[2], fz);
            if (fz == 0.0f) gz = zl; /* out of range: the copy zero-fills, = iBc * value */
            const bool pre = zl < z0, extra = zl >= z1;
            float unused = 1.0f;
            const bool split = tile_split2d || p.pmask[s2 + wrapc(zl, L2, g.bc[2], unused)];
            unsigned bytes = 4u * 3 * (TY + 2) * TEX;
            if (!pre) bytes += 4u * 3 * (TY + 1) * TQX * (split ? 3 : 2);
            if (!pre && !extra) bytes += 4u * 3 * TY * TX * (split ? 2 : 1);
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_expect(&bars[s], bytes);
            float *base = slots + s * sl.size;
            tma_load4(base + sl.e, &ft.mE, X0 - 4, Y0 - 1, gz, 3 * b, &bars[s]);
            if (pre) return;
            tma_load4(base + sl.qt, &ft.mH, X0, Y0, gz, 3 * b, &bars[s]);
            tma_load4(base + sl.qb, &ft.mBh, X0, Y0, gz, 0, &bars[s]);
            if (split) tma_load4(base + sl.qm, &ft.mHa, X0, Y0, gz, 3 * b, &bars[s]);
            if (extra) return;
            tma_load4(base + sl.be, &ft.mBe, X0, Y0, gz, 0, &bars[s]);
            if (split) tma_load4(base + sl.bm, &ft.mEa, X0, Y0, gz, 3 * b, &bars[s]);
        };

        /* after plane zl landed: the wrapped halo entries scaled by iBc = +-1 */
        auto patch = [&](int zl) {
            const int s = (zl + NS) % NS;
            float fz = 1.0f;
            const int gz = wrapc(zl, L2, g.bc[2], fz);
            const bool zw = (zl < 0 || zl >= L2) && fz != 0.0f && fz != 1.0f;
            if (!edge_tile && !zw) return;
            const long long base = pl * gz;
            const int nex = w + 2;
            for (int i = tid; i < nex * (h + 2); i += nthr) {
                const int lx = i % nex, ly = i / nex;
                float fc = fz;
                const int xx = wrapc(X0 - 1 + lx, L0, g.bc[0], fc);
                const int yy = wrapc(Y0 - 1 + ly, L1, g.bc[1], fc);
                const bool oob = xx != X0 - 1 + lx || yy != Y0 - 1 + ly;
                if (fc == 0.0f || !(oob || zw)) continue;
                const long long gi = base + xx + (long long)L0 * yy;
#pragma unroll
                for (int c = 0; c < 3; c++) TE(s, c, ly, lx + 3) = fc * Eo[c * n3 + gi];
            }
            if (zl < z0) return;
            const bool zsplit = p.pmask[s2 + gz];
            for (int i = tid; i < (w + 1) * (h + 1); i += nthr) {
                const int lx = i % (w + 1), ly = i / (w + 1);
                if (lx == w && ly == h) continue;
                float fc = fz;
                const int xx = wrapc(X0 + lx, L0, g.bc[0], fc);
                const int yy = wrapc(Y0 + ly, L1, g.bc[1], fc);
                const bool oob = xx != X0 + lx || yy != Y0 + ly;
                if (!(oob || zw)) continue;
                const long long gi = base + xx + (long long)L0 * yy;
                const bool split = zsplit || p.pmask[xx] || p.pmask[s1 + yy];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    TQ(s, sl.qt, c, ly, lx) = fc * Ho[c * n3 + gi];
                    if (oob) TQ(s, sl.qb, c, ly, lx) = p.bh[c * n3 + gi];
                    if (split) TQ(s, sl.qm, c, ly, lx) = fc * Hao[c * n3 + gi];
                }
            }
        };

        auto h_update = [&](int z, int lx, int ly, int xx, int yy, float fxy, bool split2d, float o[3], float om[3],
                            float omain[3], bool &wa) {
            wa = false;
            const int sc = (z + NS) % NS, sp = (z + NS - 1) % NS;
            float fac = fxy;
            const int gz = wrapc(z, L2, g.bc[2], fac);
            if (fac == 0.0f) {
#pragma unroll
                for (int c = 0; c < 3; c++) o[c] = om[c] = omain[c] = 0.0f;
                return;
            }
            const float c0 = TQ(sc, sl.qb, 0, ly, lx);
            if (isnan(c0)) {
                float tmp[9];
                h_general(f, b, k, xx, yy, gz, __float_as_int(TQ(sc, sl.qb, 1, ly, lx)), tmp, tmp + 3, tmp + 6);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    o[c] = tmp[c] * fac;
                    om[c] = tmp[3 + c] * fac;
                    omain[c] = tmp[6 + c] * fac;
                }
                wa = true;
                return;
            }
            const int ex = lx + 4, ey = ly + 1;
            const float Ex = TE(sc, 0, ey, ex), Ey = TE(sc, 1, ey, ex), Ez = TE(sc, 2, ey, ex);
            const float pl_[3] = {Ez - TE(sc, 2, ey - 1, ex), Ex - TE(sp, 0, ey, ex), Ey - TE(sc, 1, ey, ex - 1)};
            const float mi_[3] = {TE(sp, 1, ey, ex) - Ey, TE(sc, 2, ey, ex - 1) - Ez, TE(sc, 0, ey - 1, ex) - Ex};
            const bool split = split2d | p.pmask[s2 + gz];
            if (!split) {
                float W[3] = {pl_[0] + mi_[0], pl_[1] + mi_[1], pl_[2] + mi_[2]};
                if (gz == p.s.iI[b]) {
                    const int px = xx + L0 * yy;
                    W[0] += fac * (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, true, 1, px));
                    W[1] -= fac * (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, true, 0, px));
                }
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    o[c] = fmaf(-1.0f * TQ(sc, sl.qb, c, ly, lx), W[c], TQ(sc, sl.qt, c, ly, lx));
                    om[c] = 0.0f;
                    omain[c] = o[c];
                }
            } else {
                const int jx[3] = {xx, s1 + yy, s2 + gz};
                const float *tA = p.tab, *tG = p.tab + S;
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const int i1 = jx[(c + 1) % 3], i2 = jx[(c + 2) % 3];
                    const float bn = TQ(sc, sl.qb, c, ly, lx);
                    const float Ap = tA[i1], Bp = -1.0f * bn * tG[i1];
                    const float Am = tA[i2], Bm = -1.0f * bn * tG[i2];
                    const float m = TQ(sc, sl.qm, c, ly, lx);
                    const float pp = TQ(sc, sl.qt, c, ly, lx) - m;
                    const float np = fmaf(Bp, pl_[c], Ap * pp);
                    const float nm = fmaf(Bm, mi_[c], Am * m);
                    o[c] = np + nm;
                    om[c] = nm;
                    omain[c] = np + nm;
                }
                wa = true;
            }
        };

        bool ok = true;
        if (tid == 0) {
            issue(z0 - 1);
            for (int d = 0; d < DEPTH; d++)
                if (z0 + d <= z1) issue(z0 + d);
        }
        for (int z = z0; z <= z1; z++) {
            if (tid == 0 && z + DEPTH <= z1) issue(z + DEPTH);
            /* wait for plane z (and, on the first plane, the pre-plane z0-1) */
            const int sc = (z + NS) % NS;
            bool arrived = true;
            if (z == z0) {
                arrived = mbar_wait(&bars[(z0 - 1 + NS) % NS], 0);
                if (arrived) patch(z0 - 1);
            }
            if (arrived) arrived = mbar_wait(&bars[sc], (unsigned)(((z - (z0 - 1)) / NS) & 1));
            if (arrived) patch(z);
            ok = __syncthreads_and(arrived) != 0; /* one decision for the whole CTA */
            if (!ok) {
                if (tid == 0) atomicExch(ft.err, 1);
                /* let the copies still in flight land (bounded) before leaving */
                for (int zz = z + 1; zz <= min(z + DEPTH, z1); zz++)
                    mbar_wait(&bars[(zz + NS) % NS], (unsigned)(((zz - (z0 - 1)) / NS) & 1));
                break;
            }

            const int hs = (z - z0) % NSH;
            if (own) {
                float o[3], om[3], omain[3];
                bool wa;
                h_update(z, tx, ty, gx, gy, 1.0f, own_split2d, o, om, omain, wa);
#pragma unroll
                for (int c = 0; c < 3; c++) HN(hs, c, ty, tx) = o[c];
                if (z < z1) {
                    const long long gi = own2d + pl * z;
#pragma unroll
                    for (int c = 0; c < 3; c++) Hn[c * n3 + gi] = o[c];
                    if (wa) {
#pragma unroll
                        for (int c = 0; c < 3; c++) Han[c * n3 + gi] = om[c];
                    }
                    const int q = mon_index(p.d, z);
                    if (q >= 0) {
                        ring_ptr(p.d, g.pl, b, k, q, 0)[own2d] = omain[0];
                        ring_ptr(p.d, g.pl, b, k, q, 1)[own2d] = omain[1];
                    }
                }
            }
            if (hlx >= 0 && z < z1) {
                float o[3], om[3], omain[3];
                bool wa;
                h_update(z, hlx, hly, hxx, hyy, hfac, hsplit2d, o, om, omain, wa);
#pragma unroll
                for (int c = 0; c < 3; c++) HN(hs, c, hly, hlx) = o[c];
            }
            __syncthreads();

            if (z > z0 && own) {
                const int zp = z - 1;
                const int hp = (zp - z0) % NSH;
                const int se = (zp + NS) % NS;
                const float Hx = HN(hp, 0, ty, tx), Hy = HN(hp, 1, ty, tx), Hz = HN(hp, 2, ty, tx);
                const float pl_[3] = {HN(hp, 2, ty + 1, tx) - Hz, HN(hs, 0, ty, tx) - Hx, HN(hp, 1, ty, tx + 1) - Hy};
                const float mi_[3] = {Hy - HN(hs, 1, ty, tx), Hz - HN(hp, 2, ty, tx + 1), Hx - HN(hp, 0, ty + 1, tx)};
                const float e0[3] = {TE(se, 0, ty + 1, tx + 4), TE(se, 1, ty + 1, tx + 4), TE(se, 2, ty + 1, tx + 4)};
                const long long gi = own2d + pl * zp;
                const float c0 = TB(se, sl.be, 0);
                float eo[3], eom[3], emain[3];
                bool done = true, wa = false;
                if (!isnan(c0)) {
                    const bool split = own_split2d | p.pmask[s2 + zp];
                    if (!split) {
                        float W[3] = {pl_[0] + mi_[0], pl_[1] + mi_[1], pl_[2] + mi_[2]};
                        if (zp == p.s.iI[b]) {
                            W[0] += (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, false, 1, own2d));
                            W[1] -= (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, false, 0, own2d));
                        }
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            eo[c] = fmaf(1.0f * TB(se, sl.be, c), W[c], e0[c]);
                            emain[c] = eo[c];
                        }
                    } else {
                        const int jx[3] = {gx, s1 + gy, s2 + zp};
                        const float *tA = p.tab + 2 * S, *tG = p.tab + 3 * S;
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            const int i1 = jx[(c + 1) % 3], i2 = jx[(c + 2) % 3];
                            const float bn = TB(se, sl.be, c);
                            const float Ap = tA[i1], Bp = 1.0f * bn * tG[i1];
                            const float Am = tA[i2], Bm = 1.0f * bn * tG[i2];
                            const float m = TB(se, sl.bm, c);
                            const float pp = e0[c] - m;
                            const float np = fmaf(Bp, pl_[c], Ap * pp);
                            const float nm = fmaf(Bm, mi_[c], Am * m);
                            eo[c] = np + nm;
                            eom[c] = nm;
                            emain[c] = np + nm;
                        }
                        wa = true;
                    }
                } else {
                    const int ridx = __float_as_int(TB(se, sl.be, 1));
                    if (p.erec[ridx].kind == RK_STABLE) {
                        done = false;
                    } else {
                        float tmp[18];
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            tmp[c] = pl_[c];
                            tmp[3 + c] = mi_[c];
                            tmp[6 + c] = e0[c];
                        }
                        e_general(f, b, k, gx, gy, zp, ridx, tmp, tmp + 3, tmp + 6, tmp + 9, tmp + 12, tmp + 15);
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            eo[c] = tmp[9 + c];
                            eom[c] = tmp[12 + c];
                            emain[c] = tmp[15 + c];
                        }
                        wa = true;
                    }
                }
                if (done) {
#pragma unroll
                    for (int c = 0; c < 3; c++) En[c * n3 + gi] = eo[c];
                    if (wa) {
#pragma unroll
                        for (int c = 0; c < 3; c++) Ean[c * n3 + gi] = eom[c];
                    }
                    const int q = mon_index(p.d, zp);
                    if (q >= 0) {
                        ring_ptr(p.d, g.pl, b, k, q, 2)[own2d] = emain[0];
                        ring_ptr(p.d, g.pl, b, k, q, 3)[own2d] = emain[1];
                    }
                }
            }
        }
        if (!ok) return; /* every thread of the CTA saw the same timeout */
        __syncthreads();
    }
#undef TE
#undef TQ
#undef TB
#undef HN
}

size_t fused32t_smem(int ty, int ns) { return sizeof(float) * (32 + (size_t)ns * tslot(ty).size + (size_t)NSH * 3 * (ty + 1) * SHX); }

static void *fused_t_kernel(int ns)
{
    switch (ns) {
    case 4: return (void *)k_fused32t<4>;
    case 5: return (void *)k_fused32t<5>;
    default: return (void *)k_fused32t<6>;
    }
}

int fused32t_max_ctas_per_sm(int ty, int ns)
{
    int n = 0;
    const size_t sm = fused32t_smem(ty, ns);
    cudaFuncSetAttribute(fused_t_kernel(ns), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fused_t_kernel(ns), TX * ty, sm) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

void launch_fused32t(const Fused32T &ft, int rel, int grid, cudaStream_t st)
{
    dim3 blk(TX, ft.f.ty, 1);
    const size_t sm = fused32t_smem(ft.f.ty, ft.f.ns);
    if (ft.f.ns == 4) k_fused32t<4><<<grid, blk, sm, st>>>(ft, rel);
    else if (ft.f.ns == 5) k_fused32t<5><<<grid, blk, sm, st>>>(ft, rel);
    else k_fused32t<6><<<grid, blk, sm, st>>>(ft, rel);
    if (ft.f.nstable > 0) {
        dim3 g2((ft.f.nstable + 127) / 128, ft.f.p.batch);
        k_fix_stable32<<<g2, 128, 0, st>>>(ft.f, rel);
    }
}

} // namespace smat

namespace smat {

/* ===========================================================================
 * k_zm32: the fused step on 128 x ZNW tiles, a TMA producer warp and ZNW
 * consumer warps (kernel 5).
 *
 * Same computation and bit-identical results as the sweeps (the H and E
 * expressions of k_sweep32v per element).  Differences from k_fused32t:
 *   - a lane owns four x-cells (float4 from shared memory), so one barrier
 *     per plane covers 512 cells, not 32 x TY;
 *   - a dedicated producer warp keeps ZNS - 2 planes of TMA copies in flight
 *     ahead of the consumers (full/empty mbarriers), so the prefetch depth
 *     costs no consumer registers;
 *   - the +1 halo row and column of H_new are shared out over all consumer
 *     warps; H_new planes are triple-buffered so one named barrier per plane
 *     orders the H and E phases.
 * Plans with iBc = 0 on every axis only: the copies' zero fill outside the
 * grid is then exactly the reference's boundary factor (the fill is +0 where
 * the reference has +-0, which changes no value).  The last z chunk's extra
 * plane (z = L2) and the pre-plane -1 are fetched out of range for the same
 * reason.  Stable-form E cells are finished by k_fix_stable32.
 * ======================================================================== */
constexpr int ZTX = 128;     /* tile width: 32 lanes x 4 cells */
constexpr int ZNW = 4;       /* consumer warps = tile rows */
constexpr int ZNS = 4;       /* plane slots */
constexpr int ZEX = ZTX + 8; /* E box: x from X0-4 to X0+131 */
constexpr int ZQX = ZTX + 4; /* H, bh, Ha boxes: x from X0 to X0+131 */
constexpr int ZHX = ZTX + 4; /* H_new plane row pitch (columns 0..128 used) */
constexpr int ZNH = 3;       /* H_new planes kept */

struct ZSlot {
    int e, qt, qb, qm, be, bm, size;
};

__host__ __device__ inline ZSlot zslot()
{
    ZSlot s;
    int o = 0;
    s.e = o;
    o += align32f(3 * (ZNW + 2) * ZEX);
    s.qt = o;
    o += align32f(3 * (ZNW + 1) * ZQX);
    s.qb = o;
    o += align32f(3 * (ZNW + 1) * ZQX);
    s.qm = o;
    o += align32f(3 * (ZNW + 1) * ZQX);
    s.be = o;
    o += align32f(3 * ZNW * ZTX);
    s.bm = o;
    o += align32f(3 * ZNW * ZTX);
    s.size = o;
    return s;
}

size_t zm32_smem() { return sizeof(float) * (32 + (size_t)ZNS * zslot().size + (size_t)ZNH * 3 * (ZNW + 1) * ZHX); }

__device__ __forceinline__ void named_bar(int id, int n) { asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(n) : "memory"); }

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

/* bounded wait on phase `parity` of bar that gives up at once when another
 * warp of the CTA has already timed out (*abort): after a timeout every warp
 * still reaches every barrier, quickly, and the launch ends with the error
 * flag set instead of hanging */
__device__ __forceinline__ bool zwait(uint64_t *bar, unsigned parity, volatile int *abort, int *err)
{
    const unsigned a = smem_u32(bar);
    for (int it = 0; it < (1 << 24); it++) {
        unsigned done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (done) return true;
        if (*abort) return false;
    }
    *abort = 1;
    atomicExch(err, 3);
    return false;
}

/* work item -> (excitation, tile origin, z chunk) */
struct ZItem {
    int b, X0, Y0, z0, z1;
};

__device__ __forceinline__ ZItem zitem(const Fused32 &f, int item)
{
    ZItem it;
    it.b = item % f.p.batch;
    int t = item / f.p.batch;
    const int tix = t % f.ntx;
    t /= f.ntx;
    const int tiy = t % f.nty;
    const int zci = t / f.nty;
    it.X0 = tix * ZTX;
    it.Y0 = tiy * ZNW;
    it.z0 = zci * f.zc;
    it.z1 = min(it.z0 + f.zc, f.p.g.L2);
    return it;
}

/* does the tile (with its +-1 halo) hold a split cell in x or y? */
__device__ __forceinline__ bool ztile_split(const P32 &p, int X0, int Y0)
{
    const Geo &g = p.g;
    bool s = false;
    for (int x = max(0, X0 - 1); x <= min(g.L0 - 1, X0 + ZTX); x++) s |= p.pmask[x] != 0;
    for (int y = max(0, Y0 - 1); y <= min(g.L1 - 1, Y0 + ZNW); y++) s |= p.pmask[g.L0 + y] != 0;
    return s;
}

/* H_new of one element (cell gx, gy, gz); inputs as in k_sweep32v: h = own E
 * (x, y, z components), ey0/ey2 = Ex/Ez at y-1, ez0/ez1 = Ex/Ey at z-1,
 * nx1/nx2 = Ey/Ez at x-1; old = old total H, m = old aux, bn = coefficients.
 * Returns the new total in out, the aux in aux, and whether aux was written. */
__device__ __forceinline__ bool zm_h_elem(const Fused32 &f, int b, int k, int gx, int gy, int gz, const float h[3],
                                          float ey0, float ey2, float ez0, float ez1, float nx1, float nx2,
                                          const float bn[3], float out[3], float aux[3], float smp[2])
{
    const P32 &p = f.p;
    const Geo &g = p.g;
    if (isnan(bn[0])) { /* general cell: out of line, from the old set in global memory */
        float tmp[9];
        h_general(f, b, k, gx, gy, gz, __float_as_int(bn[1]), tmp, tmp + 3, tmp + 6);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            out[c] = tmp[c];
            aux[c] = tmp[3 + c];
        }
        smp[0] = tmp[6]; /* the DFT samples the main slot of a stable-form cell */
        smp[1] = tmp[7];
        return true;
    }
    float pl[3], mi[3];
    pl[0] = h[2] - ey2;
    mi[0] = ez1 - h[1];
    pl[1] = h[0] - ez0;
    mi[1] = nx2 - h[2];
    pl[2] = h[1] - nx1;
    mi[2] = ey0 - h[0];
    const int S = g.L0 + g.L1 + g.L2, s1 = g.L0, s2 = g.L0 + g.L1;
    const bool split = p.pmask[gx] | p.pmask[s1 + gy] | p.pmask[s2 + gz];
    if (!split) {
        float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
        if (gz == p.s.iI[b]) {
            const int px = gx + g.L0 * gy;
            W[0] += (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, true, 1, px));
            W[1] -= (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, true, 0, px));
        }
#pragma unroll
        for (int c = 0; c < 3; c++) out[c] = fmaf(-1.0f * bn[c], W[c], out[c]);
        smp[0] = out[0];
        smp[1] = out[1];
        return false;
    }
    const int jx[3] = {gx, s1 + gy, s2 + gz};
    const float *tA = p.tab, *tG = p.tab + S;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int i1 = jx[(c + 1) % 3], i2 = jx[(c + 2) % 3];
        const float Ap = tA[i1], Bp = -1.0f * bn[c] * tG[i1];
        const float Am = tA[i2], Bm = -1.0f * bn[c] * tG[i2];
        const float m = aux[c];
        const float pp = out[c] - m;
        const float np = fmaf(Bp, pl[c], Ap * pp);
        const float nm = fmaf(Bm, mi[c], Am * m);
        out[c] = np + nm;
        aux[c] = nm;
    }
    smp[0] = out[0];
    smp[1] = out[1];
    return true;
}

/* E_new of one element on plane gz: h = own H_new (x, y, z), hy0/hy2 = Hx/Hz at
 * y+1, hz0/hz1 = Hx/Hy at z+1, nx1/nx2 = Hy/Hz at x+1; out = old total E in,
 * new out.  Returns 0: plain, 1: aux written, 2: stable form (left to the
 * fix-up kernel, nothing written). */
__device__ __forceinline__ int zm_e_elem(const Fused32 &f, int b, int k, int gx, int gy, int gz, const float h[3],
                                         float hy0, float hy2, float hz0, float hz1, float nx1, float nx2,
                                         const float bn[3], float out[3], float aux[3], float smp[2])
{
    const P32 &p = f.p;
    const Geo &g = p.g;
    float pl[3], mi[3];
    pl[0] = hy2 - h[2];
    mi[0] = h[1] - hz1;
    pl[1] = hz0 - h[0];
    mi[1] = h[2] - nx2;
    pl[2] = nx1 - h[1];
    mi[2] = h[0] - hy0;
    if (isnan(bn[0])) {
        const int ridx = __float_as_int(bn[1]);
        if (p.erec[ridx].kind == RK_STABLE) return 2;
        float tmp[18];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            tmp[c] = pl[c];
            tmp[3 + c] = mi[c];
            tmp[6 + c] = out[c];
        }
        e_general(f, b, k, gx, gy, gz, ridx, tmp, tmp + 3, tmp + 6, tmp + 9, tmp + 12, tmp + 15);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            out[c] = tmp[9 + c];
            aux[c] = tmp[12 + c];
        }
        smp[0] = tmp[15];
        smp[1] = tmp[16];
        return 1;
    }
    const int S = g.L0 + g.L1 + g.L2, s1 = g.L0, s2 = g.L0 + g.L1;
    const bool split = p.pmask[gx] | p.pmask[s1 + gy] | p.pmask[s2 + gz];
    if (!split) {
        float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
        if (gz == p.s.iI[b]) {
            const int px = gx + g.L0 * gy;
            W[0] += (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, false, 1, px));
            W[1] -= (float)(p.s.sgn[b] * sheet_f(p.s, g.pl, b, k, false, 0, px));
        }
#pragma unroll
        for (int c = 0; c < 3; c++) out[c] = fmaf(1.0f * bn[c], W[c], out[c]);
        smp[0] = out[0];
        smp[1] = out[1];
        return 0;
    }
    const int jx[3] = {gx, s1 + gy, s2 + gz};
    const float *tA = p.tab + 2 * S, *tG = p.tab + 3 * S;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int i1 = jx[(c + 1) % 3], i2 = jx[(c + 2) % 3];
        const float Ap = tA[i1], Bp = 1.0f * bn[c] * tG[i1];
        const float Am = tA[i2], Bm = 1.0f * bn[c] * tG[i2];
        const float m = aux[c];
        const float pp = out[c] - m;
        const float np = fmaf(Bp, pl[c], Ap * pp);
        const float nm = fmaf(Bm, mi[c], Am * m);
        out[c] = np + nm;
        aux[c] = nm;
    }
    smp[0] = out[0];
    smp[1] = out[1];
    return 1;
}

__global__ void __launch_bounds__(32 * (ZNW + 1), 1) k_zm32(const __grid_constant__ Fused32T ft, const int rel)
{
    extern __shared__ __align__(128) float smem[];
    const Fused32 &f = ft.f;
    const P32 &p = f.p;
    const Geo &g = p.g;
    const ZSlot sl = zslot();
    uint64_t *full = reinterpret_cast<uint64_t *>(smem), *empty = full + ZNS;
    float *slots = smem + 32;
    float *hn = slots + ZNS * sl.size; /* [ZNH][3][ZNW+1][ZHX] */
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long n3 = g.n3, bs = 3 * n3, pl = g.pl;
    const int L0 = g.L0, L1 = g.L1, L2 = g.L2;
    const int s2 = L0 + L1;
    const int k = *p.s.base + rel;
#define ZE(s, c, r, x) slots[(s) * sl.size + sl.e + ((c) * (ZNW + 2) + (r)) * ZEX + (x)]
#define ZQ(s, seg, c, r, x) slots[(s) * sl.size + (seg) + ((c) * (ZNW + 1) + (r)) * ZQX + (x)]
#define ZB(s, seg, c, r, x) slots[(s) * sl.size + (seg) + ((c) * ZNW + (r)) * ZTX + (x)]
#define ZH(h, c, r, x) hn[(((h) * 3 + (c)) * (ZNW + 1) + (r)) * ZHX + (x)]
    __shared__ volatile int zabort;
    if (threadIdx.x == 0) {
        zabort = 0;
        for (int s = 0; s < ZNS; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], ZNW);
        }
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    __syncthreads();

    if (warp == ZNW) {
        /* ---------------- producer: one lane issues every copy ---------------- */
        if (lane != 0) return;
        unsigned seq = 0, issued_to = 0;
        for (int item = blockIdx.x; item < f.nitems && !zabort; item += gridDim.x) {
            const ZItem it = zitem(f, item);
            const bool tsplit = ztile_split(p, it.X0, it.Y0);
            for (int zl = it.z0 - 1; zl <= it.z1 && !zabort; zl++, seq++) {
                const int s = seq % ZNS;
                if (seq >= ZNS && !zwait(&empty[s], ((seq / ZNS) - 1) & 1, &zabort, ft.err)) break;
                issued_to = seq + 1;
                const bool pre = zl < it.z0, first = zl == it.z0;
                const bool zin = zl >= 0 && zl < L2, zpin = zl - 1 >= 0 && zl - 1 < L2;
                const bool split = tsplit || (zin && p.pmask[s2 + zl]);
                const bool bsplit = tsplit || (zpin && p.pmask[s2 + zl - 1]);
                unsigned bytes = 4u * 3 * (ZNW + 2) * ZEX;
                if (!pre) bytes += 4u * 3 * (ZNW + 1) * ZQX * (split ? 3 : 2);
                if (!pre && !first) bytes += 4u * 3 * ZNW * ZTX * (bsplit ? 2 : 1);
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                mbar_expect(&full[s], bytes);
                float *base = slots + s * sl.size;
                /* out-of-range planes (-1, L2) read as zero: iBc[2] = 0 */
                tma_load4(base + sl.e, &ft.mE, it.X0 - 4, it.Y0 - 1, zl, 3 * it.b, &full[s]);
                if (pre) continue;
                tma_load4(base + sl.qt, &ft.mH, it.X0, it.Y0, zl, 3 * it.b, &full[s]);
                tma_load4(base + sl.qb, &ft.mBh, it.X0, it.Y0, zl, 0, &full[s]);
                if (split) tma_load4(base + sl.qm, &ft.mHa, it.X0, it.Y0, zl, 3 * it.b, &full[s]);
                if (first) continue;
                tma_load4(base + sl.be, &ft.mBe, it.X0, it.Y0, zl - 1, 0, &full[s]);
                if (bsplit) tma_load4(base + sl.bm, &ft.mEa, it.X0, it.Y0, zl - 1, 3 * it.b, &full[s]);
            }
        }
        /* stay until every issued copy has landed (bounded, also after an abort) */
        for (unsigned q = (issued_to > ZNS ? issued_to - ZNS : 0); q < issued_to; q++)
            mbar_wait(&full[q % ZNS], (q / ZNS) & 1);
        return;
    }

    /* ---------------- consumers: warp = tile row, lane = four x-cells ---------------- */
    unsigned seq = 0;
    const int cx = 4 * lane; /* first column of the lane's quad in the tile */
    for (int item = blockIdx.x; item < f.nitems; item += gridDim.x) {
        const ZItem it = zitem(f, item);
        const int b = it.b;
        const int gy = it.Y0 + warp, gx0 = it.X0 + cx;
        const bool live = gy < L1 && gx0 < L0;
        const bool tsplit = ztile_split(p, it.X0, it.Y0);
        float *Hn = f.Hn + b * bs, *Han = f.Han + b * bs, *En = f.En + b * bs, *Ean = f.Ean + b * bs;
        float eprev[3][4]; /* old E of the previous plane, own quad */
        float hprev[3][4]; /* new H of the previous plane, own quad */
        for (int zl = it.z0 - 1; zl <= it.z1; zl++, seq++) {
            const int s = seq % ZNS, sp = (seq + ZNS - 1) % ZNS;
            /* after an abort the data are garbage but control flow stays uniform */
            zwait(&full[s], (seq / ZNS) & 1, &zabort, ft.err);
            __syncwarp();
            if (zl < it.z0) { /* the pre-plane: own old E of plane z0-1 */
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float4 v = lds4(&ZE(s, c, warp + 1, cx + 4));
                    eprev[c][0] = v.x, eprev[c][1] = v.y, eprev[c][2] = v.z, eprev[c][3] = v.w;
                }
                continue;
            }
            const int z = zl, hz = (z - it.z0) % ZNH, hzp = (z - it.z0 + ZNH - 1) % ZNH;
            const bool zsplit = tsplit || (z < L2 && p.pmask[s2 + z]);
            /* ---- phase A: H_new(z), own quad ---- */
            float hnew[3][4], ecur[3][4];
            {
                float e[3][4], ey[3][4], hq[3][4], bq[3][4], mq[3][4];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float4 v = lds4(&ZE(s, c, warp + 1, cx + 4));
                    e[c][0] = v.x, e[c][1] = v.y, e[c][2] = v.z, e[c][3] = v.w;
                    const float4 u = lds4(&ZE(s, c, warp, cx + 4));
                    ey[c][0] = u.x, ey[c][1] = u.y, ey[c][2] = u.z, ey[c][3] = u.w;
                    const float4 hh = lds4(&ZQ(s, sl.qt, c, warp, cx));
                    hq[c][0] = hh.x, hq[c][1] = hh.y, hq[c][2] = hh.z, hq[c][3] = hh.w;
                    const float4 bb = lds4(&ZQ(s, sl.qb, c, warp, cx));
                    bq[c][0] = bb.x, bq[c][1] = bb.y, bq[c][2] = bb.z, bq[c][3] = bb.w;
                    if (zsplit) {
                        const float4 mm = lds4(&ZQ(s, sl.qm, c, warp, cx));
                        mq[c][0] = mm.x, mq[c][1] = mm.y, mq[c][2] = mm.z, mq[c][3] = mm.w;
                    } else {
                        mq[c][0] = mq[c][1] = mq[c][2] = mq[c][3] = 0.0f;
                    }
                }
                const float xm1 = ZE(s, 1, warp + 1, cx + 3), xm2 = ZE(s, 2, warp + 1, cx + 3);
                bool wa = false;
                float smp[2][4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const float h3[3] = {e[0][i], e[1][i], e[2][i]};
                    const float bn[3] = {bq[0][i], bq[1][i], bq[2][i]};
                    float out[3] = {hq[0][i], hq[1][i], hq[2][i]}, aux[3] = {mq[0][i], mq[1][i], mq[2][i]};
                    float sm[2] = {0.0f, 0.0f};
                    const float nx1 = i == 0 ? xm1 : e[1][i - 1], nx2 = i == 0 ? xm2 : e[2][i - 1];
                    if (live && z < L2) /* elsewhere zero: inputs are zero-filled and iBc = 0 */
                        wa |= zm_h_elem(f, b, k, gx0 + i, gy, z, h3, ey[0][i], ey[2][i], eprev[0][i], eprev[1][i],
                                        nx1, nx2, bn, out, aux, sm);
                    else
                        out[0] = out[1] = out[2] = aux[0] = aux[1] = aux[2] = 0.0f;
                    smp[0][i] = sm[0];
                    smp[1][i] = sm[1];
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        hnew[c][i] = out[c];
                        mq[c][i] = aux[c];
                        ecur[c][i] = e[c][i];
                    }
                }
#pragma unroll
                for (int c = 0; c < 3; c++)
                    *reinterpret_cast<float4 *>(&ZH(hz, c, warp, cx)) =
                        make_float4(hnew[c][0], hnew[c][1], hnew[c][2], hnew[c][3]);
                if (live && z < it.z1) {
                    const long long gi = gx0 + (long long)L0 * gy + pl * z;
#pragma unroll
                    for (int c = 0; c < 3; c++)
                        *reinterpret_cast<float4 *>(Hn + c * n3 + gi) =
                            make_float4(hnew[c][0], hnew[c][1], hnew[c][2], hnew[c][3]);
                    if (wa) {
#pragma unroll
                        for (int c = 0; c < 3; c++)
                            *reinterpret_cast<float4 *>(Han + c * n3 + gi) =
                                make_float4(mq[c][0], mq[c][1], mq[c][2], mq[c][3]);
                    }
                    const int q = mon_index(p.d, z);
                    if (q >= 0) {
                        const int px = gx0 + L0 * gy;
                        *reinterpret_cast<float4 *>(ring_ptr(p.d, g.pl, b, k, q, 0) + px) =
                            make_float4(smp[0][0], smp[0][1], smp[0][2], smp[0][3]);
                        *reinterpret_cast<float4 *>(ring_ptr(p.d, g.pl, b, k, q, 1) + px) =
                            make_float4(smp[1][0], smp[1][1], smp[1][2], smp[1][3]);
                    }
                }
            }
            /* halo H_new: row ZNW (x = X0 + 4j .. +3 for the warp's 8 lanes) and
             * column ZTX (rows 0..ZNW, by lanes 8..8+ZNW of the last warp) */
            if (lane < 8 || (warp == ZNW - 1 && lane < 9 + ZNW)) {
                const bool row = lane < 8;
                const int nq = row ? 4 : 1;
                const int r = row ? ZNW : lane - 8;
                const int c0 = row ? 32 * warp + 4 * lane : ZTX;
                for (int i = 0; i < nq; i++) {
                    const int cxh = c0 + i, hx = it.X0 + cxh, hy = it.Y0 + r;
                    const float h3[3] = {ZE(s, 0, r + 1, cxh + 4), ZE(s, 1, r + 1, cxh + 4), ZE(s, 2, r + 1, cxh + 4)};
                    const float bn[3] = {ZQ(s, sl.qb, 0, r, cxh), ZQ(s, sl.qb, 1, r, cxh), ZQ(s, sl.qb, 2, r, cxh)};
                    float out[3] = {ZQ(s, sl.qt, 0, r, cxh), ZQ(s, sl.qt, 1, r, cxh), ZQ(s, sl.qt, 2, r, cxh)};
                    float aux[3] = {0.0f, 0.0f, 0.0f}, hsm[2];
                    if (zsplit) {
                        aux[0] = ZQ(s, sl.qm, 0, r, cxh);
                        aux[1] = ZQ(s, sl.qm, 1, r, cxh);
                        aux[2] = ZQ(s, sl.qm, 2, r, cxh);
                    }
                    if (hx < L0 && hy < L1 && z < L2) {
                        zm_h_elem(f, b, k, hx, hy, z, h3, ZE(s, 0, r, cxh + 4), ZE(s, 2, r, cxh + 4),
                                  ZE(sp, 0, r + 1, cxh + 4), ZE(sp, 1, r + 1, cxh + 4), ZE(s, 1, r + 1, cxh + 3),
                                  ZE(s, 2, r + 1, cxh + 3), bn, out, aux, hsm);
                    } else { /* outside the grid: iBc = 0 makes the neighbour zero */
                        out[0] = out[1] = out[2] = 0.0f;
                    }
                    ZH(hz, 0, r, cxh) = out[0];
                    ZH(hz, 1, r, cxh) = out[1];
                    ZH(hz, 2, r, cxh) = out[2];
                }
            }
            named_bar(1, 32 * ZNW);
            /* the previous plane's slot is no longer read */
            if (lane == 0) mbar_arrive(&empty[sp]);
            /* ---- phase B: E_new(z-1), own quad ---- */
            if (z > it.z0) {
                const int ze = z - 1;
                float hy[3][4], bq[3][4], mq[3][4];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float4 u = lds4(&ZH(hzp, c, warp + 1, cx));
                    hy[c][0] = u.x, hy[c][1] = u.y, hy[c][2] = u.z, hy[c][3] = u.w;
                    const float4 bb = lds4(&ZB(s, sl.be, c, warp, cx));
                    bq[c][0] = bb.x, bq[c][1] = bb.y, bq[c][2] = bb.z, bq[c][3] = bb.w;
                    const bool bsplit = tsplit || p.pmask[s2 + ze];
                    if (bsplit) {
                        const float4 mm = lds4(&ZB(s, sl.bm, c, warp, cx));
                        mq[c][0] = mm.x, mq[c][1] = mm.y, mq[c][2] = mm.z, mq[c][3] = mm.w;
                    } else {
                        mq[c][0] = mq[c][1] = mq[c][2] = mq[c][3] = 0.0f;
                    }
                }
                const float xp1 = ZH(hzp, 1, warp, cx + 4), xp2 = ZH(hzp, 2, warp, cx + 4);
                float eo[3][4], esm[2][4];
                int wa = 0, stable = 0;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const float h3[3] = {hprev[0][i], hprev[1][i], hprev[2][i]};
                    const float bn[3] = {bq[0][i], bq[1][i], bq[2][i]};
                    float out[3] = {eprev[0][i], eprev[1][i], eprev[2][i]}, aux[3] = {mq[0][i], mq[1][i], mq[2][i]};
                    const float nx1 = i == 3 ? xp1 : hprev[1][i + 1], nx2 = i == 3 ? xp2 : hprev[2][i + 1];
                    float sm[2] = {0.0f, 0.0f};
                    const int r = live ? zm_e_elem(f, b, k, gx0 + i, gy, ze, h3, hy[0][i], hy[2][i], hnew[0][i],
                                                   hnew[1][i], nx1, nx2, bn, out, aux, sm)
                                       : 0;
                    esm[0][i] = sm[0];
                    esm[1][i] = sm[1];
                    wa |= r == 1;
                    stable |= (r == 2) << i;
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        eo[c][i] = out[c];
                        mq[c][i] = aux[c];
                    }
                }
                if (live) {
                    const long long gi = gx0 + (long long)L0 * gy + pl * ze;
                    if (!stable) {
#pragma unroll
                        for (int c = 0; c < 3; c++)
                            *reinterpret_cast<float4 *>(En + c * n3 + gi) =
                                make_float4(eo[c][0], eo[c][1], eo[c][2], eo[c][3]);
                        if (wa) {
#pragma unroll
                            for (int c = 0; c < 3; c++)
                                *reinterpret_cast<float4 *>(Ean + c * n3 + gi) =
                                    make_float4(mq[c][0], mq[c][1], mq[c][2], mq[c][3]);
                        }
                    } else { /* element-wise: stable-form cells are left to k_fix_stable32 */
                        for (int i = 0; i < 4; i++) {
                            if ((stable >> i) & 1) continue;
                            for (int c = 0; c < 3; c++) {
                                En[c * n3 + gi + i] = eo[c][i];
                                if (wa) Ean[c * n3 + gi + i] = mq[c][i];
                            }
                        }
                    }
                    const int q = mon_index(p.d, ze);
                    if (q >= 0) {
                        const int px = gx0 + L0 * gy;
                        for (int i = 0; i < 4; i++) {
                            if ((stable >> i) & 1) continue;
                            ring_ptr(p.d, g.pl, b, k, q, 2)[px + i] = esm[0][i];
                            ring_ptr(p.d, g.pl, b, k, q, 3)[px + i] = esm[1][i];
                        }
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < 3; c++)
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    eprev[c][i] = ecur[c][i];
                    hprev[c][i] = hnew[c][i];
                }
        }
        /* every warp is done with this item's H_new planes before the next item
         * writes them; then the item's last slot is free */
        named_bar(1, 32 * ZNW);
        if (lane == 0) mbar_arrive(&empty[(seq + ZNS - 1) % ZNS]);
    }
#undef ZE
#undef ZQ
#undef ZB
#undef ZH
}

int zm32_max_ctas_per_sm()
{
    int n = 0;
    const size_t sm = zm32_smem();
    cudaFuncSetAttribute(k_zm32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_zm32, 32 * (ZNW + 1), sm) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

void launch_zm32(const Fused32T &ft, int rel, int grid, cudaStream_t st)
{
    const size_t sm = zm32_smem();
    k_zm32<<<grid, 32 * (ZNW + 1), sm, st>>>(ft, rel);
    if (ft.f.nstable > 0) {
        dim3 g2((ft.f.nstable + 127) / 128, ft.f.p.batch);
        k_fix_stable32<<<g2, 128, 0, st>>>(ft.f, rel);
    }
}

} // namespace smat
