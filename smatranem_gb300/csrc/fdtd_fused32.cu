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
        const float *Eo = p.E + b * bs, *Ho = p.H + b * bs, *Hao = p.Ha + b * bs, *Eao = p.Ea + b * bs;
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
