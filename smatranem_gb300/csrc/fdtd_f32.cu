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

struct Stn32 {
    long long o[3];
    float f[3]; /* boundary factor iBc at the wrapped neighbour, else 1 */
};

__device__ __forceinline__ Stn32 make_stn32(const Geo &g, int j0, int j1, int j2, bool fwd)
{
    Stn32 st;
    const int j[3] = {j0, j1, j2};
    const int L[3] = {g.L0, g.L1, g.L2};
    long long stride = 1;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const bool edge = fwd ? (j[a] + 1 == L[a]) : (j[a] == 0);
        const int jn = fwd ? (edge ? 0 : j[a] + 1) : (edge ? L[a] - 1 : j[a] - 1);
        st.o[a] = (long long)(jn - j[a]) * stride;
        st.f[a] = edge ? (float)g.bc[a] : 1.0f;
        stride *= L[a];
    }
    return st;
}

/* Half curls of a field given by an accessor get(c, offset). */
template <bool FWD, class Get>
__device__ __forceinline__ void curl32(const Get &get, const Stn32 &st, float pl[3], float mi[3])
{
    const float here[3] = {get(0, 0), get(1, 0), get(2, 0)};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        const float n2 = st.f[a1] * get(a2, st.o[a1]);
        const float n1 = st.f[a2] * get(a1, st.o[a2]);
        if (!FWD) {
            pl[c] = here[a2] - n2;
            mi[c] = n1 - here[a1];
        } else {
            pl[c] = n2 - here[a2];
            mi[c] = here[a1] - n1;
        }
    }
}

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
__global__ void __launch_bounds__(256) k_sweep32(const P32 p, const int rel)
{
    const int j0 = blockIdx.x * 32 + threadIdx.x, j1 = blockIdx.y * blockDim.y + threadIdx.y, j2 = blockIdx.z;
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
    const float c0 = cf[l];
    const long long bs = 3 * n3;

    if (!isnan(c0)) {
        const float bn[3] = {c0, cf[n3 + l], cf[2 * n3 + l]};
        const int S = g.L0 + g.L1 + g.L2, s1 = g.L0, s2 = g.L0 + g.L1;
        const Stn32 st = make_stn32(g, j0, j1, j2, EF);
        const bool split = p.pmask[j0] | p.pmask[s1 + j1] | p.pmask[s2 + j2];
        if (!split) {
            for (int b = 0; b < p.batch; b++) {
                float *F = F0 + b * bs;
                const float *G = G0 + b * bs;
                auto get = [&](int c, long long o) { return G[c * n3 + l + o]; };
                float pl[3], mi[3];
                curl32<EF>(get, st, pl, mi);
                float W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
                if (j2 == p.s.iI[b]) {
                    W[0] += (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 1, px));
                    W[1] -= (float)(p.s.sgn[b] * sheet32(p.s, g.pl, b, k, !EF, 0, px));
                }
                float f[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    f[c] = fmaf(sg * bn[c], W[c], F[c * n3 + l]);
                    F[c * n3 + l] = f[c];
                }
                if (q >= 0) {
                    ring_at(p.d, g.pl, b, k, q, EF ? 2 : 0)[px] = f[0];
                    ring_at(p.d, g.pl, b, k, q, EF ? 3 : 1)[px] = f[1];
                }
            }
        } else {
            const int jx[3] = {j0, s1 + j1, s2 + j2};
            const float *tA = p.tab + (EF ? 2 : 0) * S, *tG = p.tab + (EF ? 3 : 1) * S;
            float Ap[3], Bp[3], Am[3], Bm[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int i1 = jx[(c + 1) % 3], i2 = jx[(c + 2) % 3];
                Ap[c] = tA[i1];
                Bp[c] = sg * bn[c] * tG[i1];
                Am[c] = tA[i2];
                Bm[c] = sg * bn[c] * tG[i2];
            }
            for (int b = 0; b < p.batch; b++) {
                float *F = F0 + b * bs, *Fa = Fa0 + b * bs;
                const float *G = G0 + b * bs;
                auto get = [&](int c, long long o) { return G[c * n3 + l + o]; };
                float pl[3], mi[3];
                curl32<EF>(get, st, pl, mi);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float m = Fa[c * n3 + l];
                    const float pp = F[c * n3 + l] - m;
                    const float np = fmaf(Bp[c], pl[c], Ap[c] * pp);
                    const float nm = fmaf(Bm[c], mi[c], Am[c] * m);
                    F[c * n3 + l] = np + nm;
                    Fa[c * n3 + l] = nm;
                    if (q >= 0 && c < 2) ring_at(p.d, g.pl, b, k, q, (EF ? 2 : 0) + c)[px] = np + nm;
                }
            }
        }
        return;
    }

    /* general cells */
    const Rec32 r = (EF ? p.erec : p.hrec)[__float_as_int(cf[n3 + l])];
    const bool stable = r.kind == RK_STABLE;
    const Stn32 st = make_stn32(g, j0, j1, j2, EF && !stable);
    for (int b = 0; b < p.batch; b++) {
        float *F = F0 + b * bs, *Fa = Fa0 + b * bs;
        const float *G = G0 + b * bs, *Ga = Ga0 + b * bs;
        float main_out[3];
        if (r.kind == RK_FROZEN) {
#pragma unroll
            for (int c = 0; c < 3; c++) main_out[c] = F[c * n3 + l] - Fa[c * n3 + l];
        } else if (stable) {
            /* the stable form differentiates the MAIN slot of the other field */
            auto get = [&](int c, long long o) { return G[c * n3 + l + o] - Ga[c * n3 + l + o]; };
            float pl[3], mi[3];
            curl32<false>(get, st, pl, mi);
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
            auto get = [&](int c, long long o) { return G[c * n3 + l + o]; };
            float pl[3], mi[3];
            curl32<EF>(get, st, pl, mi);
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

/* Fold `count` ring slots ending at step *base + rel_end into the FP64 DFT
 * accumulators: acc += sum_k phase_k * x_k with an FP32 sum over the slots. */
constexpr int RING_MAX = 32;

__global__ void k_flush32(const P32 p, const int rel_end, const int count)
{
    extern __shared__ float sph[]; /* [count][nfreq][4] phases of the window */
    const Dft &d = p.d;
    const int k0 = *p.s.base + rel_end - count;
    const int nph = count * d.nfreq * 4;
    for (int i = threadIdx.x; i < nph; i += blockDim.x) {
        const int s = i / (d.nfreq * 4), r = i % (d.nfreq * 4);
        sph[i] = d.xphase32 ? d.xphase32[r & 3] : d.phase32[4 * (long long)(k0 + s) * d.nfreq + r];
    }
    __syncthreads();
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    const int qv = blockIdx.y, b = blockIdx.z;
    const int q = qv >> 2, v = qv & 3;
    if (px >= p.g.pl) return;
    float x[RING_MAX];
#pragma unroll
    for (int s = 0; s < RING_MAX; s++)
        x[s] = (s < count) ? ring_at(d, p.g.pl, b, k0 + s, q, v)[px] : 0.0f;
    const int po = v < 2 ? 0 : 2;
    for (int f = 0; f < d.nfreq; f++) {
        float sr = 0.0f, si = 0.0f;
#pragma unroll
        for (int s = 0; s < RING_MAX; s++) {
            if (s < count) {
                const float *ph = sph + (s * d.nfreq + f) * 4 + po;
                sr = fmaf(ph[0], x[s], sr);
                si = fmaf(ph[1], x[s], si);
            }
        }
        double *acc = d.acc + 2 * (((((long long)b * d.nfreq + f) * d.nq + q) * 4 + v) * p.g.pl + px);
        acc[0] += (double)sr;
        acc[1] += (double)si;
    }
}

void launch_h32(const P32 &p, int rel, int by, cudaStream_t st)
{
    dim3 blk(32, by, 1), grd((p.g.L0 + 31) / 32, (p.g.L1 + by - 1) / by, p.g.L2);
    k_sweep32<false><<<grd, blk, 0, st>>>(p, rel);
}

void launch_e32(const P32 &p, int rel, int by, cudaStream_t st)
{
    dim3 blk(32, by, 1), grd((p.g.L0 + 31) / 32, (p.g.L1 + by - 1) / by, p.g.L2);
    k_sweep32<true><<<grd, blk, 0, st>>>(p, rel);
}

void launch_flush32(const P32 &p, int rel_end, int count, cudaStream_t st)
{
    if (p.d.nfreq <= 0 || p.d.nq <= 0 || count <= 0) return;
    dim3 blk(256), grd((p.g.pl + 255) / 256, p.d.nq * 4, p.batch);
    const size_t sm = sizeof(float) * 4 * (size_t)count * p.d.nfreq;
    if (sm > 48 * 1024) cudaFuncSetAttribute(k_flush32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_flush32<<<grd, blk, sm, st>>>(p, rel_end, count);
}

} // namespace smat
