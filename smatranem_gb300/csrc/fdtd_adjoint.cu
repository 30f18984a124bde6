/*
 * Adjoint gradient of a port-overlap objective with respect to per-cell
 * permittivity: the discrete adjoint of the split-field step of a plan.
 *
 * The reference has no gradient; this is the transpose of its own update
 * (FDTDcalc/FDTDsplitfieldMetal.c main_calc :242-329), run backwards in time.
 *
 * Forward step k (per component c; main slot "+", aux slot "-" of split cells,
 * one slot for ordinary cells, whose two halves share A and B):
 *   H'+ = A+ H+ - B+ pl_c(E)      H'- = A- H- - B- mi_c(E)      (H sweep)
 *   E'+ = A+ E+ + B+ pl_c(H')     E'- = A- E- + B- mi_c(H')     (E sweep)
 * with pl/mi the two halves of the curl of the total field (backward
 * differences for H, :393-413, forward ones for E, :372-392), and a DFT sample
 * of the total H', E' on the monitor planes.  Objective
 *   J = sum_b |S_b|^2,  S_b = t_b^H x_b,  x_b = (HB_x, HB_y, -EB_y, EB_x)
 * of excitation b's DFT at one frequency and plane (the S_calc projection,
 * :437-445), with one mode column t for all excitations or one per excitation.
 *
 * Adjoint: with L = dJ/d(state) and the weighted adjoints phi+- = B+- L+- that
 * neighbours read (the transpose of "read the total" sends the same value to
 * both slots), one backward step k is
 *   phi_E+- <- A+- phi_E+- + B+- s_E,  s_E,c = -(pl_c(psi_H) + mi_c(phi_H)) + g_E,c
 *   phi_H+- <- A+- phi_H+- + B+- s_H,  s_H,c = +(pl_c(psi_E) + mi_c(phi_E)) + g_H,c
 * where pl/mi keep the stencil of the forward E (resp. H) sweep -- the
 * transpose of the backward-difference curl is the forward-difference curl --
 * but read psi = phi- in the "+" term and phi = phi+ in the "-" term, and g is
 * the objective's sensitivity to the DFT sample of step k.  Scaling a cell's
 * permittivity by (1 + s) scales its E coefficient B to B/(1 + s) (A is a ratio
 * and stays), so dJ/ds = -sum_k sum_c L_E,c^{k+1} (E_c^{k+1} - A E_c^k).
 *
 * Time reversal of the forward fields is unstable through the PML, so the
 * forward pass keeps a checkpoint of the whole state every K steps and each
 * backward segment recomputes its K forward steps from the checkpoint,
 * recording E on the design cells only.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "trace.cuh"
#include "plan_internal.cuh"

using namespace smat;
using namespace smat::plan;

namespace smat {
namespace adj {

template <class T> struct AState {
    T *phiH, *psiH, *phiE, *psiE; /* [batch][3][n3] */
};

struct Obj {
    int zq;               /* z index of the monitor plane */
    int f, nfreq;
    const double *phase;  /* [nsched][nfreq][4]: H re, im, E re, im */
    const double2 *ad;    /* [batch][4][pl]: conj(S_b) * sign * conj(t) per DFT component */
};

struct Box {
    int x0, y0, z0, nx, ny, nz;
    long long n;
};

/* coefficients of one cell and component of an FP32 plan, exactly as its
 * forward kernels use them */
struct Coef32 {
    const float *bh, *be;
    const Rec32 *hrec, *erec;
    const float *tab;
    const uint8_t *pmask;
    int S, s1, s2;

    __device__ void get(bool efield, int c, long long l, long long n3, int x, int y, int z, float &Ap, float &Bp,
                        float &Am, float &Bm) const
    {
        const float *cf = efield ? be : bh;
        if (isnan(cf[l])) {
            const Rec32 r = (efield ? erec : hrec)[__float_as_int(cf[n3 + l])];
            Ap = r.A0[c];
            Bp = r.B0[c];
            if (r.kind == RK_A) {
                Am = r.A1[c];
                Bm = r.B1[c];
            } else {
                Am = Ap;
                Bm = Bp;
            }
            return;
        }
        const float bn = cf[c * n3 + l];
        if (!(pmask[x] | pmask[s1 + y] | pmask[s2 + z])) {
            Ap = Am = 1.0f;
            Bp = Bm = bn;
            return;
        }
        const int jx[3] = {x, s1 + y, s2 + z};
        const int i1 = jx[(c + 1) % 3], i2 = jx[(c + 2) % 3];
        const float *tA = tab + (efield ? 2 * S : 0), *tG = tab + (efield ? 3 * S : S);
        Ap = tA[i1];
        Bp = bn * tG[i1];
        Am = tA[i2];
        Bm = bn * tG[i2];
    }
};

/* the same for an FP64 plan: main coefficients per cell, aux ones per slot */
struct Coef64 {
    const uint8_t *flags;
    const int *addr;
    const double *cm, *ca;
    int lnotn;

    __device__ void get(bool efield, int c, long long l, long long n3, int, int, int, double &Ap, double &Bp,
                        double &Am, double &Bm) const
    {
        const int wA = efield ? 2 : 0, wB = wA + 1;
        Ap = cm[((long long)wA * 3 + c) * n3 + l];
        Bp = cm[((long long)wB * 3 + c) * n3 + l];
        if ((flags[l] & 7) == CLS_A) {
            const long long a = addr[l];
            Am = ca[((long long)wA * 3 + c) * lnotn + a];
            Bm = ca[((long long)wB * 3 + c) * lnotn + a];
        } else {
            Am = Ap;
            Bm = Bp;
        }
    }
};

__device__ __forceinline__ bool in_box(const Box &bx, int x, int y, int z, long long &i)
{
    const int u = x - bx.x0, v = y - bx.y0, w = z - bx.z0;
    if (u < 0 || v < 0 || w < 0 || u >= bx.nx || v >= bx.ny || w >= bx.nz) return false;
    i = u + (long long)bx.nx * (v + (long long)bx.ny * w);
    return true;
}

/* objective sensitivity to the DFT sample v (0, 1: H_x, H_y; 2, 3: E_x, E_y)
 * of step k at pixel px of excitation b */
__device__ __forceinline__ double sample_sens(const Obj &o, int b, int v, int px, int pl, int k)
{
    const double *ph = o.phase + 4 * ((long long)k * o.nfreq + o.f) + (v < 2 ? 0 : 2);
    const double2 a = o.ad[((long long)b * 4 + v) * pl + px];
    return 2.0 * (a.x * ph[0] - a.y * ph[1]);
}

/* transpose of the E sweep of step k; also accumulates the design gradient
 * -L_E^{k+1} (E^{k+1} - A E^k) on the box cells ([batch][3][nbox]) */
template <class T, class C>
__global__ void __launch_bounds__(256) k_adj_e(const Geo g, const int batch, const C coef, const AState<T> s,
                                               const Obj o, const int k, const Box bx, const T *__restrict__ rec1,
                                               const T *__restrict__ rec0, double *__restrict__ grad)
{
    const long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (l >= g.n3) return;
    const long long n3 = g.n3, bs = 3 * n3;
    const int x = (int)(l % g.L0), y = (int)((l / g.L0) % g.L1), z = (int)(l / g.pl);
    const T *PH = s.phiH + b * bs, *QH = s.psiH + b * bs;
    T *PE = s.phiE + b * bs, *QE = s.psiE + b * bs;
    const int j[3] = {x, y, z}, L[3] = {g.L0, g.L1, g.L2};
    long long o_[3];
    T f[3];
    long long stride = 1;
#pragma unroll
    for (int a = 0; a < 3; a++) { /* forward neighbour along a, wrapped with iBc */
        const bool edge = j[a] + 1 == L[a];
        o_[a] = (edge ? -(long long)(L[a] - 1) : 1LL) * stride;
        f[a] = edge ? (T)g.bc[a] : (T)1;
        stride *= L[a];
    }
    T gs[2] = {0, 0};
    if (z == o.zq) {
        const int px = x + g.L0 * y;
        gs[0] = (T)sample_sens(o, b, 2, px, g.pl, k);
        gs[1] = (T)sample_sens(o, b, 3, px, g.pl, k);
    }
    long long bi = 0;
    const bool design = grad && in_box(bx, x, y, z, bi);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        const T pl_ = f[a1] * QH[a2 * n3 + l + o_[a1]] - QH[a2 * n3 + l];
        const T mi_ = PH[a1 * n3 + l] - f[a2] * PH[a1 * n3 + l + o_[a2]];
        const T sv = -(pl_ + mi_) + (c < 2 ? gs[c] : (T)0);
        T Ap, Bp, Am, Bm;
        coef.get(true, c, l, n3, x, y, z, Ap, Bp, Am, Bm);
        const T phi = Ap * PE[c * n3 + l] + Bp * sv;
        PE[c * n3 + l] = phi;
        QE[c * n3 + l] = Am * QE[c * n3 + l] + Bm * sv;
        if (design && Bp != (T)0) {
            const long long r = ((long long)b * 3 + c) * bx.n + bi;
            const double lam = (double)phi / (double)Bp;
            grad[r] -= lam * ((double)rec1[r] - (double)Ap * (double)rec0[r]);
        }
    }
}

/* transpose of the H sweep of step k */
template <class T, class C>
__global__ void __launch_bounds__(256) k_adj_h(const Geo g, const int batch, const C coef, const AState<T> s,
                                               const Obj o, const int k)
{
    const long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (l >= g.n3) return;
    const long long n3 = g.n3, bs = 3 * n3;
    const int x = (int)(l % g.L0), y = (int)((l / g.L0) % g.L1), z = (int)(l / g.pl);
    T *PH = s.phiH + b * bs, *QH = s.psiH + b * bs;
    const T *PE = s.phiE + b * bs, *QE = s.psiE + b * bs;
    const int j[3] = {x, y, z}, L[3] = {g.L0, g.L1, g.L2};
    long long o_[3];
    T f[3];
    long long stride = 1;
#pragma unroll
    for (int a = 0; a < 3; a++) { /* backward neighbour along a, wrapped with iBc */
        const bool edge = j[a] == 0;
        o_[a] = (edge ? (long long)(L[a] - 1) : -1LL) * stride;
        f[a] = edge ? (T)g.bc[a] : (T)1;
        stride *= L[a];
    }
    T gs[2] = {0, 0};
    if (z == o.zq) {
        const int px = x + g.L0 * y;
        gs[0] = (T)sample_sens(o, b, 0, px, g.pl, k);
        gs[1] = (T)sample_sens(o, b, 1, px, g.pl, k);
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        const T pl_ = QE[a2 * n3 + l] - f[a1] * QE[a2 * n3 + l + o_[a1]];
        const T mi_ = -PE[a1 * n3 + l] + f[a2] * PE[a1 * n3 + l + o_[a2]];
        const T sv = pl_ + mi_ + (c < 2 ? gs[c] : (T)0);
        T Ap, Bp, Am, Bm;
        coef.get(false, c, l, n3, x, y, z, Ap, Bp, Am, Bm);
        PH[c * n3 + l] = Ap * PH[c * n3 + l] + Bp * sv;
        QH[c * n3 + l] = Am * QH[c * n3 + l] + Bm * sv;
    }
}

/* E of the design cells: dst[b][c][i] = E[b][c][cell i] */
template <class T>
__global__ void k_adj_record(const Geo g, const int batch, const Box bx, const T *__restrict__ E, T *__restrict__ dst)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (i >= bx.n) return;
    const int u = (int)(i % bx.nx), v = (int)((i / bx.nx) % bx.ny), w = (int)(i / ((long long)bx.nx * bx.ny));
    const long long l = (bx.x0 + u) + (long long)g.L0 * ((bx.y0 + v) + (long long)g.L1 * (bx.z0 + w));
#pragma unroll
    for (int c = 0; c < 3; c++) dst[((long long)b * 3 + c) * bx.n + i] = E[((long long)b * 3 + c) * g.n3 + l];
}

/* ---------------------------------------------------------------------------
 * Vectorised FP32 adjoint steps (L0 % 4 == 0): four x-cells per thread, as
 * the forward sweep k_sweep32v -- float4 loads of the adjoint fields and the
 * coefficient stream, x neighbours by warp shuffle -- with the per-element
 * arithmetic of k_adj_e / k_adj_h.  A block is 32 x by threads; grid as
 * k_sweep32v's (x blocks, row blocks x excitations, planes).
 * ------------------------------------------------------------------------- */
__device__ __forceinline__ float4 ldf4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void stf4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float e4(const float4 &v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }
__device__ __forceinline__ void s4(float4 &v, int i, float x)
{
    if (i == 0) v.x = x;
    else if (i == 1) v.y = x;
    else if (i == 2) v.z = x;
    else v.w = x;
}

/* coefficients (A+, B+, A-, B-) of component c of element i of a quad whose
 * coefficient stream components are cq[3] (same rules as Coef32::get) */
__device__ __forceinline__ void coef32_elem(const Coef32 &cf, bool efield, const float4 cq[3], int i, int c,
                                            bool split, int x, int y, int z, float &Ap, float &Bp, float &Am,
                                            float &Bm)
{
    const float c0 = e4(cq[0], i);
    if (isnan(c0)) {
        const Rec32 r = (efield ? cf.erec : cf.hrec)[__float_as_int(e4(cq[1], i))];
        Ap = r.A0[c];
        Bp = r.B0[c];
        if (r.kind == RK_A) {
            Am = r.A1[c];
            Bm = r.B1[c];
        } else {
            Am = Ap;
            Bm = Bp;
        }
        return;
    }
    const float bn = e4(cq[c], i);
    if (!split) {
        Ap = Am = 1.0f;
        Bp = Bm = bn;
        return;
    }
    const int jx[3] = {x, cf.s1 + y, cf.s2 + z};
    const int i1 = jx[(c + 1) % 3], i2 = jx[(c + 2) % 3];
    const float *tA = cf.tab + (efield ? 2 * cf.S : 0), *tG = cf.tab + (efield ? 3 * cf.S : cf.S);
    Ap = tA[i1];
    Bp = bn * tG[i1];
    Am = tA[i2];
    Bm = bn * tG[i2];
}

template <bool EF>
__global__ void __launch_bounds__(128, 4) k_adj32v(const Geo g, const int batch, const Coef32 cf,
                                                  const AState<float> s, const Obj o, const int k, const Box bx,
                                                  const float *__restrict__ rec1, const float *__restrict__ rec0,
                                                  double *__restrict__ grad)
{
    const int b = blockIdx.y % batch;
    const int xr = (blockIdx.x * 32 + threadIdx.x) * 4;
    const int y = (blockIdx.y / batch) * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (y >= g.L1) return; /* uniform per warp */
    const bool live = xr < g.L0;
    const int x0 = live ? xr : g.L0 - 4;
    const long long n3 = g.n3, bs = 3 * n3;
    const long long l = x0 + (long long)g.L0 * (y + (long long)g.L1 * z);
    /* EF: transpose of the E sweep (reads the H adjoint, forward neighbours);
     * else of the H sweep (reads the E adjoint, backward neighbours) */
    const float *PG = (EF ? s.phiH : s.phiE) + b * bs, *QG = (EF ? s.psiH : s.psiE) + b * bs;
    float *PF = (EF ? s.phiE : s.phiH) + b * bs, *QF = (EF ? s.psiE : s.psiH) + b * bs;
    const float *cfs = EF ? cf.be : cf.bh;
    const bool ey = EF ? (y + 1 == g.L1) : (y == 0);
    const bool ez = EF ? (z + 1 == g.L2) : (z == 0);
    const long long oy = (long long)g.L0 * (EF ? (ey ? -(g.L1 - 1) : 1) : (ey ? g.L1 - 1 : -1));
    const long long oz = (long long)g.pl * (EF ? (ez ? -(g.L2 - 1) : 1) : (ez ? g.L2 - 1 : -1));
    const float fy = ey ? (float)g.bc[1] : 1.0f, fz = ez ? (float)g.bc[2] : 1.0f;
    /* In a quad with no split cell psi equals phi: both start at zero and take
     * the same coefficients (A- = A+, B- = B+) and the same source.  Such quads
     * neither read nor write psi, and neighbours read their phi in its place;
     * psi is kept (read and written) for quads with a split cell only. */
    const bool pmx = cf.pmask[x0] | cf.pmask[x0 + 1] | cf.pmask[x0 + 2] | cf.pmask[x0 + 3];
    const bool pmy = cf.pmask[cf.s1 + y], pmz = cf.pmask[cf.s2 + z];
    const bool qsplit = pmx | pmy | pmz;
    const int yn = EF ? (ey ? 0 : y + 1) : (ey ? g.L1 - 1 : y - 1);
    const int zn = EF ? (ez ? 0 : z + 1) : (ez ? g.L2 - 1 : z - 1);
    const bool ysplit = pmx | cf.pmask[cf.s1 + yn] | pmz, zsplit = pmx | pmy | cf.pmask[cf.s2 + zn];
    float4 cq[3], pf[3], qf[3], pg[3], qg[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        cq[c] = ldf4(cfs + c * n3 + l);
        pf[c] = ldf4(PF + c * n3 + l);
        pg[c] = ldf4(PG + c * n3 + l);
    }
    if (qsplit) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            qf[c] = ldf4(QF + c * n3 + l);
            qg[c] = ldf4(QG + c * n3 + l);
        }
    } else {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            qf[c] = pf[c];
            qg[c] = pg[c];
        }
    }
    /* y and z neighbours: EF reads psi_z, phi_x at y+1 and phi_y, psi_x at z+1;
     * the H transpose reads psi_z, phi_x at y-1 and phi_y, psi_x at z-1 */
    float4 qyz = ldf4((ysplit ? QG : PG) + 2 * n3 + l + oy), pyx = ldf4(PG + 0 * n3 + l + oy);
    float4 pzy = ldf4(PG + 1 * n3 + l + oz), qzx = ldf4((zsplit ? QG : PG) + 0 * n3 + l + oz);
    /* x neighbours: phi_z and psi_y at x+1 (EF) or x-1 */
    const unsigned full = 0xffffffffu;
    float xpz, xqy;
    if (EF) {
        xpz = __shfl_down_sync(full, pg[2].x, 1);
        xqy = __shfl_down_sync(full, qg[1].x, 1);
        if ((threadIdx.x & 31) == 31 || x0 + 4 == g.L0) {
            const bool edge = x0 + 4 == g.L0;
            const long long ox = edge ? -(g.L0 - 4) : 4;
            const float f = edge ? (float)g.bc[0] : 1.0f;
            const int xq = edge ? 0 : x0 + 4; /* the neighbouring quad */
            const bool xsplit = pmy | pmz | cf.pmask[xq] | cf.pmask[xq + 1] | cf.pmask[xq + 2] | cf.pmask[xq + 3];
            xpz = f * PG[2 * n3 + l + ox];
            xqy = f * (xsplit ? QG : PG)[1 * n3 + l + ox];
        }
    } else {
        xpz = __shfl_up_sync(full, pg[2].w, 1);
        xqy = __shfl_up_sync(full, qg[1].w, 1);
        if ((threadIdx.x & 31) == 0 || x0 == 0) {
            const bool edge = x0 == 0;
            const long long ox = edge ? g.L0 - 1 : -1;
            const float f = edge ? (float)g.bc[0] : 1.0f;
            const int xq = edge ? g.L0 - 4 : x0 - 4; /* the neighbouring quad */
            const bool xsplit = pmy | pmz | cf.pmask[xq] | cf.pmask[xq + 1] | cf.pmask[xq + 2] | cf.pmask[xq + 3];
            xpz = f * PG[2 * n3 + l + ox];
            xqy = f * (xsplit ? QG : PG)[1 * n3 + l + ox];
        }
    }
    if (!live) return;
    const float fx_in = 1.0f;
    const bool pyzm = pmy | pmz;
    float gs[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    if (z == o.zq) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int px = x0 + i + g.L0 * y;
            gs[0][i] = (float)sample_sens(o, b, EF ? 2 : 0, px, g.pl, k);
            gs[1][i] = (float)sample_sens(o, b, EF ? 3 : 1, px, g.pl, k);
        }
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int x = x0 + i;
        const bool split = cf.pmask[x] | pyzm;
        /* neighbour along x of element i: phi_z, psi_y */
        const float npz = EF ? (i == 3 ? xpz : e4(pg[2], i + 1)) : (i == 0 ? xpz : e4(pg[2], i - 1));
        const float nqy = EF ? (i == 3 ? xqy : e4(qg[1], i + 1)) : (i == 0 ? xqy : e4(qg[1], i - 1));
        float sv[3];
        if (EF) { /* -(pl + mi), forward neighbours */
            const float pl0 = fy * e4(qyz, i) - e4(qg[2], i), mi0 = e4(pg[1], i) - fz * e4(pzy, i);
            const float pl1 = fz * e4(qzx, i) - e4(qg[0], i), mi1 = e4(pg[2], i) - fx_in * npz;
            const float pl2 = fx_in * nqy - e4(qg[1], i), mi2 = e4(pg[0], i) - fy * e4(pyx, i);
            sv[0] = -(pl0 + mi0) + gs[0][i];
            sv[1] = -(pl1 + mi1) + gs[1][i];
            sv[2] = -(pl2 + mi2);
        } else { /* +(pl + mi), backward neighbours */
            const float pl0 = e4(qg[2], i) - fy * e4(qyz, i), mi0 = -e4(pg[1], i) + fz * e4(pzy, i);
            const float pl1 = e4(qg[0], i) - fz * e4(qzx, i), mi1 = -e4(pg[2], i) + fx_in * npz;
            const float pl2 = e4(qg[1], i) - fx_in * nqy, mi2 = -e4(pg[0], i) + fy * e4(pyx, i);
            sv[0] = pl0 + mi0 + gs[0][i];
            sv[1] = pl1 + mi1 + gs[1][i];
            sv[2] = pl2 + mi2;
        }
        long long bi = 0;
        const bool design = EF && grad && in_box(bx, x, y, z, bi);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            float Ap, Bp, Am, Bm;
            coef32_elem(cf, EF, cq, i, c, split, x, y, z, Ap, Bp, Am, Bm);
            const float phi = Ap * e4(pf[c], i) + Bp * sv[c];
            s4(pf[c], i, phi);
            s4(qf[c], i, Am * e4(qf[c], i) + Bm * sv[c]);
            if (design && Bp != 0.0f) {
                const long long r = ((long long)b * 3 + c) * bx.n + bi;
                const double lam = (double)phi / (double)Bp;
                grad[r] -= lam * ((double)rec1[r] - (double)Ap * (double)rec0[r]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) stf4(PF + c * n3 + l, pf[c]);
    if (qsplit) {
#pragma unroll
        for (int c = 0; c < 3; c++) stf4(QF + c * n3 + l, qf[c]);
    }
}

} // namespace adj
} // namespace smat

using namespace smat::adj;

namespace {

/* device buffers of one adjoint call, freed on every return path */
struct Scratch {
    std::vector<void *> bufs;
    cudaStream_t st = nullptr;
    template <class T> int get(T **p, size_t n)
    {
        int rc = dalloc(p, n, st);
        if (rc == SMAT_OK && *p) bufs.push_back(*p);
        return rc;
    }
    ~Scratch()
    {
        if (st) cudaStreamSynchronize(st);
        for (void *b : bufs) cudaFree(b);
    }
};

/* the arrays that make up the state of a plan (current field set) */
struct StateView {
    void *ptr[4];
    size_t bytes[4];
};

StateView state_view(smat_fdtd_plan *p)
{
    StateView v;
    const size_t b = (size_t)p->batch;
    if (p->precision == SMAT_FP64) {
        v.ptr[0] = p->d_H64;
        v.ptr[1] = p->d_E64;
        v.ptr[2] = p->d_Ha64;
        v.ptr[3] = p->d_Ea64;
        v.bytes[0] = v.bytes[1] = b * 3 * p->n3 * 8;
        v.bytes[2] = v.bytes[3] = b * 3 * (size_t)(p->lnotn + 1) * 8;
    } else {
        const P32 q = make_p32(p, false);
        v.ptr[0] = q.H;
        v.ptr[1] = q.E;
        v.ptr[2] = q.Ha;
        v.ptr[3] = q.Ea;
        v.bytes[0] = v.bytes[1] = v.bytes[2] = v.bytes[3] = b * 3 * p->n3 * 4;
    }
    return v;
}

int zero_state(smat_fdtd_plan *p)
{
    drop_graph(p);
    p->cur = 0;
    if (p->precision == SMAT_FP64) {
        StateView v = state_view(p);
        for (int i = 0; i < 4; i++) CK(cudaMemsetAsync(v.ptr[i], 0, v.bytes[i], p->stream));
    } else {
        const size_t n = (size_t)p->batch * 3 * p->n3 * 4;
        float *arrs[8] = {p->d_H32, p->d_E32, p->d_Ha32, p->d_Ea32, p->d_H32b, p->d_E32b, p->d_Ha32b, p->d_Ea32b};
        for (float *a : arrs)
            if (a) CK(cudaMemsetAsync(a, 0, n, p->stream));
        if (p->d_ring)
            CK(cudaMemsetAsync(p->d_ring, 0, (size_t)p->batch * RING_K * p->nq * 4 * p->pl * 4, p->stream));
    }
    if (p->d_acc)
        CK(cudaMemsetAsync(p->d_acc, 0, (size_t)p->batch * p->nfreq * p->nq * 4 * p->pl * 2 * 8, p->stream));
    return SMAT_OK;
}

/* the vectorised FP32 adjoint step where it applies (L0 % 4 == 0); false:
 * the caller launches the scalar kernels */
bool adj_launch_vec(smat_fdtd_plan *p, const Geo &g, int batch, const Coef32 &cf, const AState<float> &as,
                    const Obj &o, int k, const Box &bx, const float *rec1, const float *rec0, double *grad)
{
    if (g.L0 % 4 != 0 || p->adj_scalar) return false;
    const int by = 2;
    const dim3 blk(32, by, 1), grd((g.L0 / 4 + 31) / 32, ((g.L1 + by - 1) / by) * batch, g.L2);
    k_adj32v<true><<<grd, blk, 0, p->stream>>>(g, batch, cf, as, o, k, bx, rec1, rec0, grad);
    k_adj32v<false><<<grd, blk, 0, p->stream>>>(g, batch, cf, as, o, k, bx, nullptr, nullptr, nullptr);
    return true;
}

bool adj_launch_vec(smat_fdtd_plan *, const Geo &, int, const Coef64 &, const AState<double> &, const Obj &, int,
                    const Box &, const double *, const double *, double *)
{
    return false;
}

template <class T, class C>
int adjoint_run(smat_fdtd_plan *p, const C &coef, int nsteps, int K, int f, int q, int ncols, const double *tcols,
                const Box &bx, double *grad, double *grad_c, double *J)
{
    Scratch sc;
    sc.st = p->stream;
    const long long n3 = p->n3;
    const int batch = p->batch, pl = p->pl;
    const int nseg = (nsteps + K - 1) / K;
    StateView sv = state_view(p);
    size_t ck_bytes = 0;
    for (int i = 0; i < 4; i++) ck_bytes += sv.bytes[i];
    const size_t fs = (size_t)batch * 3 * n3;
    const size_t rec_n = (size_t)batch * 3 * bx.n;
    const size_t need = ck_bytes * nseg + 4 * fs * sizeof(T) + rec_n * sizeof(T) * (K + 1) + rec_n * 8;
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    if (need > fr / 10 * 9)
        return smat_fail(SMAT_ENOMEM, "adjoint: %zu bytes of checkpoints and adjoint state, %zu free (raise K)", need,
                         fr);
    int rc;
    char *ckpt = nullptr;
    T *phiH, *psiH, *phiE, *psiE, *rec;
    double *dgrad;
    double2 *dad;
    if ((rc = sc.get(&ckpt, ck_bytes * nseg))) return rc;
    if ((rc = sc.get(&phiH, fs)) || (rc = sc.get(&psiH, fs)) || (rc = sc.get(&phiE, fs)) || (rc = sc.get(&psiE, fs)))
        return rc;
    if ((rc = sc.get(&rec, rec_n * (K + 1))) || (rc = sc.get(&dgrad, rec_n))) return rc;
    if ((rc = sc.get(&dad, (size_t)batch * 4 * pl))) return rc;

    /* ---- forward pass from rest, checkpoint every K steps ---- */
    if ((rc = zero_state(p))) return rc;
    {
        smat::TraceRange trace_fwd("adjoint: forward with checkpoints");
        for (int j = 0; j < nseg; j++) {
            sv = state_view(p);
            size_t off = ck_bytes * j;
            for (int i = 0; i < 4; i++) {
                CK(cudaMemcpyAsync(ckpt + off, sv.ptr[i], sv.bytes[i], cudaMemcpyDeviceToDevice, p->stream));
                off += sv.bytes[i];
            }
            const int k0 = j * K, k1 = k0 + K < nsteps ? k0 + K : nsteps;
            if ((rc = smat_fdtd_run(p, k0, k1))) return rc;
        }
        if ((rc = smat_fdtd_sync(p))) return rc;
    }

    /* ---- objective and its sensitivity to the DFT samples ---- */
    const int zq = p->planes[q];
    std::vector<double> acc(8 * (size_t)pl), adh(8 * (size_t)pl * batch);
    double Jv = 0.0;
    for (int b = 0; b < batch; b++) {
        if ((rc = smat_fdtd_get_dft(p, b, f, q, acc.data()))) return rc;
        const double *tcol = tcols + (ncols == 1 ? 0 : (size_t)b * 8 * pl); /* 4*pl complex per column */
        std::complex<double> S = 0.0;
        /* rows of t: HB_x, HB_y, -EB_y, EB_x; DFT components v: H_x, H_y, E_x, E_y */
        const int row_of_v[4] = {0, 1, 3, 2};
        const double sgn_of_v[4] = {1.0, 1.0, 1.0, -1.0};
        for (int v = 0; v < 4; v++)
            for (int px = 0; px < pl; px++) {
                const std::complex<double> t(tcol[2 * ((size_t)row_of_v[v] * pl + px)],
                                             tcol[2 * ((size_t)row_of_v[v] * pl + px) + 1]);
                const std::complex<double> x(acc[2 * ((size_t)v * pl + px)], acc[2 * ((size_t)v * pl + px) + 1]);
                S += std::conj(t) * sgn_of_v[v] * x;
            }
        Jv += std::norm(S);
        for (int v = 0; v < 4; v++)
            for (int px = 0; px < pl; px++) {
                const std::complex<double> t(tcol[2 * ((size_t)row_of_v[v] * pl + px)],
                                             tcol[2 * ((size_t)row_of_v[v] * pl + px) + 1]);
                const std::complex<double> a = std::conj(S) * sgn_of_v[v] * std::conj(t);
                const size_t i = ((size_t)b * 4 + v) * pl + px;
                adh[2 * i] = a.real();
                adh[2 * i + 1] = a.imag();
            }
    }
    *J = Jv;
    CK(cudaMemcpyAsync(dad, adh.data(), adh.size() * 8, cudaMemcpyHostToDevice, p->stream));

    /* ---- backward pass: per segment, recompute then adjoint ---- */
    smat::TraceRange trace_bwd("adjoint: recompute and backward");
    const Geo g = make_geo(p);
    const Obj o{zq, f, p->nfreq, p->d_phase, dad};
    const AState<T> as{phiH, psiH, phiE, psiE};
    const dim3 gc((unsigned)((n3 + 255) / 256), batch), gr((unsigned)((bx.n + 255) / 256), batch);
    const int nq_save = p->nq;
    p->nq = 0; /* no DFT sampling while recomputing */
    drop_graph(p);
    for (int j = nseg - 1; j >= 0 && rc == SMAT_OK; j--) {
        const int k0 = j * K, k1 = k0 + K < nsteps ? k0 + K : nsteps;
        sv = state_view(p);
        size_t off = ck_bytes * j;
        for (int i = 0; i < 4; i++) {
            if (cudaMemcpyAsync(sv.ptr[i], ckpt + off, sv.bytes[i], cudaMemcpyDeviceToDevice, p->stream) !=
                cudaSuccess)
                rc = smat_fail(SMAT_ECUDA, "adjoint: checkpoint restore");
            off += sv.bytes[i];
        }
        launch_set(p->d_base, k0, p->stream);
        k_adj_record<T><<<gr, 256, 0, p->stream>>>(g, batch, bx, (const T *)state_view(p).ptr[1], rec);
        for (int k = k0; k < k1; k++) {
            enqueue_steps(p, k - k0, 1, false);
            k_adj_record<T><<<gr, 256, 0, p->stream>>>(g, batch, bx, (const T *)state_view(p).ptr[1],
                                                        rec + rec_n * (k - k0 + 1));
        }
        for (int k = k1 - 1; k >= k0; k--) {
            if (adj_launch_vec(p, g, batch, coef, as, o, k, bx, rec + rec_n * (k - k0 + 1), rec + rec_n * (k - k0),
                               dgrad))
                continue;
            k_adj_e<T, C><<<gc, 256, 0, p->stream>>>(g, batch, coef, as, o, k, bx, rec + rec_n * (k - k0 + 1),
                                                     rec + rec_n * (k - k0), dgrad);
            k_adj_h<T, C><<<gc, 256, 0, p->stream>>>(g, batch, coef, as, o, k);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_fail(e, "adjoint: launch");
    }
    p->nq = nq_save;
    drop_graph(p);
    if (rc) return rc;
    std::vector<double> hg(rec_n);
    CK(cudaMemcpyAsync(hg.data(), dgrad, rec_n * 8, cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    for (long long i = 0; i < bx.n; i++) {
        double sum = 0.0;
        for (int c = 0; c < 3; c++) {
            double sc_ = 0.0;
            for (int b = 0; b < batch; b++) sc_ += hg[((size_t)b * 3 + c) * bx.n + i];
            if (grad_c) grad_c[c * bx.n + i] = sc_;
            sum += sc_;
        }
        grad[i] = sum;
    }
    return SMAT_OK;
}

} // namespace

extern "C" int smat_fdtd_adjoint_grad(smat_fdtd_plan *p, int nsteps, int K, int f, int q, int ncols, const double *tilXi_cols,
                                      const int box[6], double *grad, double *grad_c, double *J)
{
    smat_clear_error();
    if (!p || !tilXi_cols || !box || !grad || !J) return smat_fail(SMAT_EINVAL, "adjoint: null argument");
    if (ncols != 1 && ncols != p->batch)
        return smat_fail(SMAT_EINVAL, "adjoint: %d objective columns: give 1 or one per excitation (%d)", ncols,
                         p->batch);
    if (nsteps < 1 || nsteps > p->nsched || !p->d_sched)
        return smat_fail(SMAT_EINVAL, "adjoint: nsteps %d outside the %d-step schedule", nsteps, p->nsched);
    if (K < 1) return smat_fail(SMAT_EINVAL, "adjoint: checkpoint interval K must be >= 1");
    if (f < 0 || f >= p->nfreq || q < 0 || q >= p->nq || !p->d_phase)
        return smat_fail(SMAT_EINVAL, "adjoint: frequency %d / plane %d not in the DFT schedule", f, q);
    Box bx;
    bx.x0 = box[0];
    bx.y0 = box[2];
    bx.z0 = box[4];
    bx.nx = box[1] - box[0];
    bx.ny = box[3] - box[2];
    bx.nz = box[5] - box[4];
    if (bx.x0 < 0 || bx.y0 < 0 || bx.z0 < 0 || bx.nx < 1 || bx.ny < 1 || bx.nz < 1 || box[1] > p->L[0] ||
        box[3] > p->L[1] || box[5] > p->L[2])
        return smat_fail(SMAT_EINVAL, "adjoint: design box [%d,%d)x[%d,%d)x[%d,%d) outside the grid", box[0], box[1],
                         box[2], box[3], box[4], box[5]);
    bx.n = (long long)bx.nx * bx.ny * bx.nz;
    for (long long l = 0; l < p->n3; l++) {
        const char k = p->cont[l];
        if (k == 'h' || k == 'e' || k == 'b')
            return smat_fail(SMAT_EINVAL, "adjoint: cell %lld is a stable-form (metal) cell; not supported", l);
    }
    for (int w = 0; w < bx.nz; w++)
        for (int v = 0; v < bx.ny; v++)
            for (int u = 0; u < bx.nx; u++) {
                const long long l = (bx.x0 + u) + (long long)p->L[0] * ((bx.y0 + v) + (long long)p->L[1] * (bx.z0 + w));
                if (p->cont[l] != 'n')
                    return smat_fail(SMAT_EINVAL, "adjoint: design cell %lld is a PML cell", l);
            }
    if (p->precision == SMAT_FP32) {
        /* SMATRAN_ADJOINT_SCALAR=1: the one-cell-per-thread kernels even where
         * the vectorised ones apply (for comparing the two) */
        const char *sc = getenv("SMATRAN_ADJOINT_SCALAR");
        p->adj_scalar = sc && sc[0] && sc[0] != '0';
        Coef32 c;
        c.bh = p->d_bh;
        c.be = p->d_be;
        c.hrec = p->d_hrec;
        c.erec = p->d_erec;
        c.tab = p->d_tab;
        c.pmask = p->d_pmask;
        c.S = p->L[0] + p->L[1] + p->L[2];
        c.s1 = p->L[0];
        c.s2 = p->L[0] + p->L[1];
        return adjoint_run<float>(p, c, nsteps, K, f, q, ncols, tilXi_cols, bx, grad, grad_c, J);
    }
    Coef64 c;
    c.flags = p->d_flags;
    c.addr = p->d_addr;
    c.cm = p->d_cm;
    c.ca = p->d_ca;
    c.lnotn = p->lnotn;
    return adjoint_run<double>(p, c, nsteps, K, f, q, ncols, tilXi_cols, bx, grad, grad_c, J);
}
