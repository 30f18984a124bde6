/*
 * Dense complex FP64 linear algebra on the GPU for the layer-transfer S matrix
 * (Smat/Scalc.c inv_process :316-400, which calls LAPACK zgesv and BLAS
 * zgemm): a blocked right-looking LU with partial pivoting, the solve with
 * many right-hand sides, a general multiply-add and a transpose.  Column-major
 * storage with leading dimensions, as LAPACK keeps it.
 *
 * The sizes are those of the transfer: order NA = 2*L0*L1 (a few thousand at
 * most: Scalc's matrices are dense NA x NA), so every step is compute bound in
 * FP64 and the tiled multiply-add carries the O(NA^3) work.  The panel
 * factorisation runs in one CTA (NA x 32 complex values, L2 resident).
 */
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "dense_z.cuh"
#include "host_internal.h"
#include "smatran_fdtd.h"

namespace smat {
namespace dense {

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cfms(double2 c, double2 a, double2 b)  // c - a*b
{
    return make_double2(c.x - (a.x * b.x - a.y * b.y), c.y - (a.x * b.y + a.y * b.x));
}
__device__ __forceinline__ double2 crecip(double2 a)
{
    const double d = a.x * a.x + a.y * a.y;
    return make_double2(a.x / d, -a.y / d);
}

/* ---- C += alpha * A * B (m x n, inner k), tiles of 64 x 64, 256 threads with
 * 4 x 4 outputs each, k staged 16 at a time in shared memory ------------- */
constexpr int TM = 64, TN = 64, TK = 16;

__global__ void __launch_bounds__(256) k_zgemm(int m, int n, int k, double2 alpha, const double2 *__restrict__ A,
                                               int lda, const double2 *__restrict__ B, int ldb, double2 *C, int ldc)
{
    __shared__ double2 As[TK][TM + 1];
    __shared__ double2 Bs[TK][TN + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;
    double2 acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = make_double2(0.0, 0.0);
    for (int k0 = 0; k0 < k; k0 += TK) {
        for (int t = threadIdx.x; t < TK * TM; t += 256) {  // A tile: rows m0.., cols k0..
            const int r = t % TM, c = t / TM;
            const int gr = m0 + r, gc = k0 + c;
            As[c][r] = (gr < m && gc < k) ? A[gr + (long long)lda * gc] : make_double2(0.0, 0.0);
        }
        for (int t = threadIdx.x; t < TK * TN; t += 256) {  // B tile: rows k0.., cols n0..
            const int r = t % TK, c = t / TK;
            const int gr = k0 + r, gc = n0 + c;
            Bs[r][c] = (gr < k && gc < n) ? B[gr + (long long)ldb * gc] : make_double2(0.0, 0.0);
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < TK; kk++) {
            double2 a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    acc[i][j].x = fma(a[i].x, b[j].x, fma(-a[i].y, b[j].y, acc[i][j].x));
                    acc[i][j].y = fma(a[i].x, b[j].y, fma(a[i].y, b[j].x, acc[i][j].y));
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int gr = m0 + tx + 16 * i, gc = n0 + ty + 16 * j;
            if (gr < m && gc < n) {
                double2 *c = C + gr + (long long)ldc * gc;
                const double2 v = cmul(alpha, acc[i][j]);
                *c = make_double2(c->x + v.x, c->y + v.y);
            }
        }
}

int zgemm_acc(int m, int n, int k, double2 alpha, const double2 *A, int lda, const double2 *B, int ldb, double2 *C,
              int ldc, const GemmCtx *g, cudaStream_t st)
{
    if (m <= 0 || n <= 0 || k <= 0) return SMAT_OK;
    if (g && g->tc) return zgemm_acc_tc(m, n, k, alpha, A, lda, B, ldb, C, ldc, *g, st);
    const dim3 grid((unsigned)((m + TM - 1) / TM), (unsigned)((n + TN - 1) / TN));
    k_zgemm<<<grid, 256, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, C, ldc);
    return cudaPeekAtLastError() == cudaSuccess ? SMAT_OK : smat_fail(SMAT_ECUDA, "k_zgemm launch");
}

/* ---- out (n x m) = in^T (in: m x n), optionally conjugated -------------- */
__global__ void k_transpose(int m, int n, const double2 *__restrict__ in, int ldi, double2 *__restrict__ out, int ldo,
                            int conj)
{
    __shared__ double2 t[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int r = bx + threadIdx.x, c = by + j;
        if (r < m && c < n) t[j][threadIdx.x] = in[r + (long long)ldi * c];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int r = by + threadIdx.x, c = bx + j;  // out row r (= in column), out column c (= in row)
        if (r < n && c < m) {
            double2 v = t[threadIdx.x][j];
            if (conj) v.y = -v.y;
            out[r + (long long)ldo * c] = v;
        }
    }
}

int transpose(int m, int n, const double2 *in, int ldi, double2 *out, int ldo, bool conj, cudaStream_t st)
{
    if (m <= 0 || n <= 0) return SMAT_OK;
    const dim3 grid((unsigned)((m + 31) / 32), (unsigned)((n + 31) / 32));
    k_transpose<<<grid, dim3(32, 8), 0, st>>>(m, n, in, ldi, out, ldo, conj ? 1 : 0);
    return cudaPeekAtLastError() == cudaSuccess ? SMAT_OK : smat_fail(SMAT_ECUDA, "k_transpose launch");
}

/* ---- panel factorisation: rows [0, m) x columns [0, nb) of the panel at A
 * (the trailing part of the matrix from the current diagonal), partial
 * pivoting by |re| + |im| (LAPACK's izamax), first maximum on ties.
 * ipiv[c] receives the absolute pivot row row0 + p; *info the first zero
 * pivot (1-based, absolute) if any. */
constexpr int PT = 512;

__global__ void __launch_bounds__(PT) k_panel(double2 *A, int lda, int m, int nb, int row0, int *ipiv, int *info)
{
    __shared__ double sv[PT];
    __shared__ int si[PT];
    __shared__ int piv_s;
    for (int c = 0; c < nb && c < m; c++) {
        double best = -1.0;
        int bi = m;
        for (int r = c + threadIdx.x; r < m; r += PT) {
            const double2 a = A[r + (long long)lda * c];
            const double v = fabs(a.x) + fabs(a.y);
            if (v > best) {
                best = v;
                bi = r;
            }
        }
        sv[threadIdx.x] = best;
        si[threadIdx.x] = bi;
        __syncthreads();
        for (int h = PT / 2; h > 0; h >>= 1) {
            if (threadIdx.x < h) {
                const double v2 = sv[threadIdx.x + h];
                const int i2 = si[threadIdx.x + h];
                if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
                    sv[threadIdx.x] = v2;
                    si[threadIdx.x] = i2;
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            const int p = si[0] < m ? si[0] : c;
            piv_s = p;
            ipiv[c] = row0 + p;
            if (sv[0] == 0.0 && *info == 0) *info = row0 + c + 1;
        }
        __syncthreads();
        const int p = piv_s;
        if (p != c)
            for (int j = threadIdx.x; j < nb; j += PT) {
                const double2 t = A[c + (long long)lda * j];
                A[c + (long long)lda * j] = A[p + (long long)lda * j];
                A[p + (long long)lda * j] = t;
            }
        __syncthreads();
        const double2 d = A[c + (long long)lda * c];
        if (d.x != 0.0 || d.y != 0.0) {
            const double2 inv = crecip(d);
            for (int r = c + 1 + threadIdx.x; r < m; r += PT) A[r + (long long)lda * c] = cmul(A[r + (long long)lda * c], inv);
        }
        __syncthreads();
        /* rank-1 update of the panel's remaining columns */
        const int rows = m - c - 1, cols = nb - c - 1;
        for (long long t = threadIdx.x; t < (long long)rows * cols; t += PT) {
            const int r = c + 1 + (int)(t % rows), j = c + 1 + (int)(t / rows);
            A[r + (long long)lda * j] = cfms(A[r + (long long)lda * j], A[r + (long long)lda * c], A[c + (long long)lda * j]);
        }
        __syncthreads();
    }
}

constexpr int NBMAX = 32;

/* X (nb x ncols at X, leading dimension ldx) <- T^{-1} X with T the nb x nb
 * triangle at T (unit lower if lower, else non-unit upper, nb <= 32): one
 * warp per column, lane r holds x_r; the triangle is staged column by column
 * in shared memory (lane r reads entry r of a column: conflict-free) with the
 * reciprocals of its diagonal, and step k broadcasts x_k by shuffle.  The FP64
 * work of many columns is spread over every SM (the FP64 rate of one SM is a
 * few multiply-adds per clock). */
constexpr int TW = 8; /* warps (columns) per block */
__device__ __forceinline__ double2 shfl2(double2 v, int src)
{
    return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
__global__ void __launch_bounds__(TW * 32) k_trsm_w(const double2 *__restrict__ T, int ldt, int nb, double2 *X,
                                                    int ldx, int ncols, int lower)
{
    __shared__ double2 tcol[NBMAX][NBMAX]; /* tcol[k][r] = T[r][k] */
    __shared__ double2 rdiag[NBMAX];       /* 1 / T[k][k] (upper) */
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
        const int r = t % nb, k = t / nb;
        tcol[k][r] = T[r + (long long)ldt * k];
    }
    if (!lower && threadIdx.x < nb) rdiag[threadIdx.x] = crecip(T[threadIdx.x + (long long)ldt * threadIdx.x]);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int col = blockIdx.x * TW + (threadIdx.x >> 5);
    if (col >= ncols) return;
    double2 *xc = X + (long long)ldx * col;
    double2 x = lane < nb ? xc[lane] : make_double2(0.0, 0.0);
    if (lower) {
        for (int k = 0; k + 1 < nb; k++) {
            const double2 xk = shfl2(x, k);
            if (lane > k && lane < nb) x = cfms(x, tcol[k][lane], xk);
        }
    } else {
        for (int k = nb - 1; k >= 0; k--) {
            if (lane == k) x = cmul(x, rdiag[k]);
            const double2 xk = shfl2(x, k);
            if (lane < k) x = cfms(x, tcol[k][lane], xk);
        }
    }
    if (lane < nb) xc[lane] = x;
}

/* ---- panel factorisation by a thread-block cluster ----------------------
 * The m x nb panel (nb <= 32) is spread over the CTAs of one cluster, rows
 * [rank R, rank R + R) each, in shared memory; the rows are never moved: a
 * permutation (pos: logical position of each physical row, lrow: its
 * inverse, the same on every CTA) records the interchanges, and the rows go
 * back to their final positions at the end.  Per column c: each CTA's largest
 * |re| + |im| among its rows at logical positions >= c (ties: the smaller
 * logical position, as izamax's first maximum) goes to a slot in its shared
 * memory (two slot sets, by column parity); one cluster barrier; every CTA
 * reads the slots and the pivot row (distributed shared memory; a pivoted row
 * is never written again), updates the permutation, scales its rows below the
 * pivot and applies the rank-1 update -- the operations of k_panel on every
 * element, in the same order, so the same bits. */
struct PivSlot {
    double v;
    int lpos, phys;
};
constexpr int PCT = 256; /* threads per CTA */

__global__ void __launch_bounds__(PCT) k_panel_cl(double2 *A, int lda, int m, int nb, int row0, int *ipiv, int *info)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int nc = (int)cl.num_blocks(), rank = (int)cl.block_rank();
    const int R = (m + nc - 1) / nc, rbeg = rank * R, rn = max(0, min(m, rbeg + R) - rbeg);
    extern __shared__ __align__(16) unsigned char psm[];
    double2 *a = reinterpret_cast<double2 *>(psm);          /* [R][NBMAX] */
    double2 *prow = a + (size_t)R * NBMAX;                   /* the pivot row */
    PivSlot *slot = reinterpret_cast<PivSlot *>(prow + NBMAX); /* [2] */
    int *pos = reinterpret_cast<int *>(slot + 2);            /* [m] */
    int *lrow = pos + m;                                     /* [m] */
    __shared__ double rv[PCT / 32];
    __shared__ int rp[PCT / 32], rq[PCT / 32];
    __shared__ int piv_q, piv_l;
    __shared__ double piv_v;
    __shared__ double2 piv_inv;
    const int tid = threadIdx.x;
    for (int t = tid; t < rn * nb; t += PCT) {
        const int i = t % rn, j = t / rn;
        a[i * NBMAX + j] = A[(rbeg + i) + (long long)lda * j];
    }
    for (int r = tid; r < m; r += PCT) pos[r] = lrow[r] = r;
    cl.sync();
    for (int c = 0; c < nb && c < m; c++) {
        /* this CTA's candidate: a warp reduction, then one over the warps */
        double best = -1.0;
        int bl = m, bq = -1;
        for (int i = tid; i < rn; i += PCT) {
            const int lp = pos[rbeg + i];
            if (lp < c) continue;
            const double2 v = a[i * NBMAX + c];
            const double s = fabs(v.x) + fabs(v.y);
            if (s > best || (s == best && lp < bl)) {
                best = s;
                bl = lp;
                bq = rbeg + i;
            }
        }
        auto better = [](double v2, int l2, double v, int l) { return v2 > v || (v2 == v && l2 < l); };
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double v2 = __shfl_xor_sync(0xffffffffu, best, o);
            const int l2 = __shfl_xor_sync(0xffffffffu, bl, o), q2 = __shfl_xor_sync(0xffffffffu, bq, o);
            if (better(v2, l2, best, bl)) {
                best = v2;
                bl = l2;
                bq = q2;
            }
        }
        if ((tid & 31) == 0) {
            rv[tid >> 5] = best;
            rp[tid >> 5] = bl;
            rq[tid >> 5] = bq;
        }
        __syncthreads();
        if (tid < 32) {
            best = tid < PCT / 32 ? rv[tid] : -1.0;
            bl = tid < PCT / 32 ? rp[tid] : m;
            bq = tid < PCT / 32 ? rq[tid] : -1;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double v2 = __shfl_xor_sync(0xffffffffu, best, o);
                const int l2 = __shfl_xor_sync(0xffffffffu, bl, o), q2 = __shfl_xor_sync(0xffffffffu, bq, o);
                if (better(v2, l2, best, bl)) {
                    best = v2;
                    bl = l2;
                    bq = q2;
                }
            }
            if (tid == 0) {
                rv[0] = best;
                rp[0] = bl;
                rq[0] = bq;
            }
        }
        __syncthreads();
        if (tid == 0) slot[c & 1] = PivSlot{rv[0], rp[0], rq[0]};
        cl.sync();
        /* the cluster's pivot: warp 0 reads the slots */
        if (tid < 32) {
            PivSlot s{-1.0, m, -1};
            if (tid < nc) s = *cl.map_shared_rank(slot + (c & 1), tid);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double v2 = __shfl_xor_sync(0xffffffffu, s.v, o);
                const int l2 = __shfl_xor_sync(0xffffffffu, s.lpos, o);
                const int q2 = __shfl_xor_sync(0xffffffffu, s.phys, o);
                if (v2 > s.v || (v2 == s.v && l2 < s.lpos)) {
                    s.v = v2;
                    s.lpos = l2;
                    s.phys = q2;
                }
            }
            if (tid == 0) {
                /* no candidate at all cannot happen for c < m; a zero column
                 * keeps the diagonal (izamax returns the first index) */
                int q = s.phys, lq = s.lpos;
                if (q < 0) {
                    q = lrow[c];
                    lq = c;
                }
                piv_q = q;
                piv_l = lq;
                piv_v = s.v;
            }
        }
        __syncthreads();
        const int q = piv_q, lq = piv_l;
        if (tid < nb) {
            const int o = q / R;
            const double2 *src = cl.map_shared_rank(a, o);
            prow[tid] = src[(q - o * R) * NBMAX + tid];
        }
        if (tid == 32) { /* the pivot's reciprocal, once (another warp than the bookkeeping) */
            const int o = q / R;
            const double2 d = cl.map_shared_rank(a, o)[(q - o * R) * NBMAX + c];
            piv_inv = (d.x != 0.0 || d.y != 0.0) ? crecip(d) : make_double2(0.0, 0.0);
        }
        if (tid == 0) {
            if (rank == 0) {
                ipiv[c] = row0 + lq;
                if (piv_v == 0.0 && *info == 0) *info = row0 + c + 1;
            }
            const int lc = lrow[c];
            pos[lc] = lq;
            lrow[lq] = lc;
            pos[q] = c;
            lrow[c] = q;
        }
        __syncthreads();
        /* scale the column below the pivot, then the rank-1 update */
        const double2 d = prow[c];
        const bool sc = d.x != 0.0 || d.y != 0.0;
        const double2 inv = piv_inv;
        if (sc)
            for (int i = tid; i < rn; i += PCT)
                if (pos[rbeg + i] > c) a[i * NBMAX + c] = cmul(a[i * NBMAX + c], inv);
        __syncthreads();
        const int w = nb - c - 1;
        if (w > 0)
            for (int t = tid; t < rn * w; t += PCT) {
                const int i = t / w, j = c + 1 + t % w;
                if (pos[rbeg + i] > c) a[i * NBMAX + j] = cfms(a[i * NBMAX + j], a[i * NBMAX + c], prow[j]);
            }
        __syncthreads();
    }
    /* every row to its final (logical) position */
    for (int t = tid; t < rn * nb; t += PCT) {
        const int i = t % rn, j = t / rn;
        A[pos[rbeg + i] + (long long)lda * j] = a[i * NBMAX + j];
    }
    cl.sync(); /* no CTA leaves while another may still read its rows */
}

/* the cluster form for an m-row panel: cluster size (16, else 8) and shared
 * memory, or 0 where it does not fit (the one-CTA k_panel then) */
static int panel_cluster(int m, size_t *smem)
{
    /* the cluster size (16, else 8) and the shared-memory limit in KB, found
     * once per process (thread-safe initialisation: passes of smat_scalc may
     * run on two host threads) */
    static const int cached = [] {
        int c = 0, dev = 0, optin = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess &&
            cudaFuncSetAttribute(k_panel_cl, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
            cudaFuncSetAttribute(k_panel_cl, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - 8192) == cudaSuccess) {
            for (int cs : {16, 8}) {
                cudaLaunchConfig_t cfg = {};
                cudaLaunchAttribute at[1];
                at[0].id = cudaLaunchAttributeClusterDimension;
                at[0].val.clusterDim.x = cs;
                at[0].val.clusterDim.y = 1;
                at[0].val.clusterDim.z = 1;
                cfg.gridDim = dim3(cs);
                cfg.blockDim = dim3(PCT);
                cfg.dynamicSmemBytes = 96 * 1024;
                cfg.attrs = at;
                cfg.numAttrs = 1;
                int n = 0;
                if (cudaOccupancyMaxActiveClusters(&n, k_panel_cl, &cfg) == cudaSuccess && n > 0) {
                    c = cs;
                    break;
                }
            }
            c = c * 100000 + (optin - 8192) / 1024;
        }
        cudaGetLastError();
        return c;
    }();
    const int cs = cached / 100000;
    const size_t limit = (size_t)(cached % 100000) * 1024;
    if (cs == 0) return 0;
    const int R = (m + cs - 1) / cs;
    const size_t need = sizeof(double2) * ((size_t)R * NBMAX + NBMAX) + 2 * sizeof(PivSlot) + 2 * sizeof(int) * (size_t)m;
    if (need > limit || need > 200 * 1024) return 0;
    *smem = need;
    return cs;
}

static int launch_panel(double2 *A, int lda, int m, int nb, int row0, int *ipiv, int *info, cudaStream_t st)
{
    size_t smem = 0;
    const int cs = panel_cluster(m, &smem);
    if (cs == 0 || m < 2 * cs) {
        k_panel<<<1, PT, 0, st>>>(A, lda, m, nb, row0, ipiv, info);
        return cudaPeekAtLastError() == cudaSuccess ? SMAT_OK : smat_fail(SMAT_ECUDA, "k_panel launch");
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(PCT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k_panel_cl, A, lda, m, nb, row0, ipiv, info) != cudaSuccess)
        return smat_fail(SMAT_ECUDA, "k_panel_cl launch: %s", cudaGetErrorString(cudaGetLastError()));
    return SMAT_OK;
}

/* Row interchanges ipiv[k0..k1) (absolute rows, k1 - k0 <= 32) applied in
 * order to the columns [c0, c1) of A: their net permutation of the (at most
 * 64) rows they touch, built once per block, then one warp per column reads
 * every touched row and writes it to its destination (the stores wait for all
 * of the warp's loads: no row is overwritten before it is read). */
constexpr int LW = 8; /* warps (columns) per block */
__global__ void __launch_bounds__(LW * 32) k_laswp_w(double2 *A, int lda, int c0, int c1, const int *__restrict__ ipiv,
                                                    int k0, int k1)
{
    __shared__ int rows[2 * NBMAX], src[2 * NBMAX];
    __shared__ int nrows;
    if (threadIdx.x == 0) {
        int n = 0;
        for (int k = k0; k < k1; k++) {
            const int p = ipiv[k];
            if (p == k) continue;
            int a = -1, b = -1;
            for (int i = 0; i < n; i++) {
                if (rows[i] == k) a = i;
                if (rows[i] == p) b = i;
            }
            if (a < 0) {
                rows[n] = k;
                src[n] = k;
                a = n++;
            }
            if (b < 0) {
                rows[n] = p;
                src[n] = p;
                b = n++;
            }
            const int t = src[a]; /* src[i]: the original row now held by rows[i] */
            src[a] = src[b];
            src[b] = t;
        }
        nrows = n;
    }
    __syncthreads();
    const int n = nrows, lane = threadIdx.x & 31;
    const int c = c0 + blockIdx.x * LW + (threadIdx.x >> 5);
    if (c >= c1 || n == 0) return;
    double2 *col = A + (long long)lda * c;
    double2 v0 = make_double2(0.0, 0.0), v1 = v0;
    if (lane < n) v0 = col[src[lane]];
    if (lane + 32 < n) v1 = col[src[lane + 32]];
    if (lane < n) col[rows[lane]] = v0;
    if (lane + 32 < n) col[rows[lane + 32]] = v1;
}

static int launch_ok(const char *what)
{
    return cudaPeekAtLastError() == cudaSuccess ? SMAT_OK : smat_fail(SMAT_ECUDA, "%s launch", what);
}

int getrf(int n, double2 *A, int lda, int *ipiv, int *info, const GemmCtx *g, cudaStream_t st)
{
    const double2 m1 = make_double2(-1.0, 0.0);
    for (int j = 0; j < n; j += NBMAX) {
        const int nb = std::min(NBMAX, n - j);
        if (int rc = launch_panel(A + j + (long long)lda * j, lda, n - j, nb, j, ipiv + j, info, st)) return rc;
        /* the panel's pivots are local to rows [j, n): make them absolute is done
         * in k_panel (row0 = j); apply them left and right of the panel */
        if (j > 0) {
            k_laswp_w<<<(j + LW - 1) / LW, LW * 32, 0, st>>>(A, lda, 0, j, ipiv, j, j + nb);
            if (int rc = launch_ok("k_laswp_w")) return rc;
        }
        const int right = n - j - nb;
        if (right > 0) {
            k_laswp_w<<<(right + LW - 1) / LW, LW * 32, 0, st>>>(A, lda, j + nb, n, ipiv, j, j + nb);
            if (int rc = launch_ok("k_laswp_w")) return rc;
            k_trsm_w<<<(right + TW - 1) / TW, TW * 32, 0, st>>>(A + j + (long long)lda * j, lda, nb,
                                                                A + j + (long long)lda * (j + nb), lda, right, 1);
            if (int rc = launch_ok("k_trsm_w")) return rc;
            if (int rc = zgemm_acc(n - j - nb, right, nb, m1, A + (j + nb) + (long long)lda * j, lda,
                                   A + j + (long long)lda * (j + nb), lda, A + (j + nb) + (long long)lda * (j + nb),
                                   lda, g, st))
                return rc;
        }
    }
    return SMAT_OK;
}

int getrs(int n, int nrhs, const double2 *LU, int lda, const int *ipiv, double2 *B, int ldb, const GemmCtx *g,
          cudaStream_t st)
{
    if (n <= 0 || nrhs <= 0) return SMAT_OK;
    const double2 m1 = make_double2(-1.0, 0.0);
    for (int j = 0; j < n; j += NBMAX) { /* the interchanges of each panel, in order */
        k_laswp_w<<<(nrhs + LW - 1) / LW, LW * 32, 0, st>>>(B, ldb, 0, nrhs, ipiv, j, std::min(n, j + NBMAX));
        if (int rc = launch_ok("k_laswp_w")) return rc;
    }
    for (int j = 0; j < n; j += NBMAX) {  // L y = b
        const int nb = std::min(NBMAX, n - j);
        k_trsm_w<<<(nrhs + TW - 1) / TW, TW * 32, 0, st>>>(LU + j + (long long)lda * j, lda, nb, B + j, ldb, nrhs, 1);
        if (int rc = launch_ok("k_trsm_w")) return rc;
        if (int rc = zgemm_acc(n - j - nb, nrhs, nb, m1, LU + (j + nb) + (long long)lda * j, lda, B + j, ldb,
                               B + j + nb, ldb, g, st))
            return rc;
    }
    for (int j = ((n - 1) / NBMAX) * NBMAX; j >= 0; j -= NBMAX) {  // U x = y
        const int nb = std::min(NBMAX, n - j);
        k_trsm_w<<<(nrhs + TW - 1) / TW, TW * 32, 0, st>>>(LU + j + (long long)lda * j, lda, nb, B + j, ldb, nrhs, 0);
        if (int rc = launch_ok("k_trsm_w")) return rc;
        if (int rc = zgemm_acc(j, nrhs, nb, m1, LU + (long long)lda * j, lda, B + j, ldb, B, ldb, g, st)) return rc;
    }
    return SMAT_OK;
}

} // namespace dense
} // namespace smat

/* ---- process-wide mode and test hooks -------------------------------------- */

namespace smat {
namespace dense {
static int g_mode = 1;
int dense_mode() { return g_mode; }

/* a context for products up to m x n: the tensor-core workspace and error
 * flag on the device when mode 1 is chosen and the device runs it (freed by
 * release) */
int gemm_ctx_alloc(GemmCtx &g, int m, int n, cudaStream_t st)
{
    g = GemmCtx{0, nullptr, 0, nullptr, 0, -1};
    if (dense_mode() != 1 || !tc_available()) return SMAT_OK;
    g.ws_bytes = tc_workspace_bytes(m, n);
    if (cudaMalloc(&g.ws, g.ws_bytes) != cudaSuccess || cudaMalloc(&g.err, sizeof(int)) != cudaSuccess ||
        cudaMemsetAsync(g.err, 0, sizeof(int), st) != cudaSuccess) {
        gemm_ctx_release(g);
        return smat_fail(SMAT_ENOMEM, "dense: tensor-core workspace of %zu bytes", g.ws_bytes);
    }
    g.tc = 1;
    return SMAT_OK;
}

/* after the stream is synchronised: SMAT_ECUDA if a tensor-core product gave
 * up waiting for its operands */
int gemm_ctx_check(const GemmCtx &g)
{
    if (!g.tc) return SMAT_OK;
    int e = 0;
    if (cudaMemcpy(&e, g.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return smat_fail(SMAT_ECUDA, "dense: error flag read");
    return e ? smat_fail(SMAT_ECUDA, "dense: tensor-core product timed out waiting (%d)", e) : SMAT_OK;
}

void gemm_ctx_release(GemmCtx &g)
{
    cudaFree(g.ws);
    cudaFree(g.err);
    g = GemmCtx{0, nullptr, 0, nullptr, 0, -1};
}

} // namespace dense
} // namespace smat

extern "C" int smat_dense_mode(int mode)
{
    if (mode != 0 && mode != 1) return smat_fail(SMAT_EINVAL, "smat_dense_mode: %d (0: FP64 kernel, 1: tensor cores)", mode);
    smat::dense::g_mode = mode;
    return SMAT_OK;
}

extern "C" int smat_zgesv(int n, int nrhs, const double *A, const double *B, double *X, int *info_out)
{
    using namespace smat::dense;
    if (n <= 0 || nrhs <= 0 || !A || !B || !X) return smat_fail(SMAT_EINVAL, "smat_zgesv: n = %d, nrhs = %d", n, nrhs);
    cudaStream_t st = nullptr;
    double2 *dA = nullptr, *dB = nullptr;
    int *dp = nullptr, *dinfo = nullptr;
    int rc = SMAT_OK, info = 0;
    GemmCtx g{0, nullptr, 0, nullptr, 0, -1};
    const size_t an = (size_t)n * n, bn = (size_t)n * nrhs;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&dA, an * sizeof(double2)) != cudaSuccess || cudaMalloc(&dB, bn * sizeof(double2)) != cudaSuccess ||
        cudaMalloc(&dp, (size_t)n * sizeof(int)) != cudaSuccess || cudaMalloc(&dinfo, sizeof(int)) != cudaSuccess)
        rc = smat_fail(SMAT_ENOMEM, "smat_zgesv: device allocation");
    if (!rc) rc = gemm_ctx_alloc(g, n, n > nrhs ? n : nrhs, st);
    if (!rc && (cudaMemcpyAsync(dA, A, an * sizeof(double2), cudaMemcpyHostToDevice, st) != cudaSuccess ||
                cudaMemcpyAsync(dB, B, bn * sizeof(double2), cudaMemcpyHostToDevice, st) != cudaSuccess ||
                cudaMemsetAsync(dinfo, 0, sizeof(int), st) != cudaSuccess))
        rc = smat_fail(SMAT_ECUDA, "smat_zgesv: upload");
    if (!rc) rc = getrf(n, dA, n, dp, dinfo, &g, st);
    if (!rc) rc = getrs(n, nrhs, dA, n, dp, dB, n, &g, st);
    if (!rc && (cudaMemcpyAsync(X, dB, bn * sizeof(double2), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = smat_fail(SMAT_ECUDA, "smat_zgesv: %s", cudaGetErrorString(cudaGetLastError()));
    if (!rc) rc = gemm_ctx_check(g);
    if (info_out) *info_out = info;
    if (st) cudaStreamSynchronize(st);
    gemm_ctx_release(g);
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dp);
    cudaFree(dinfo);
    if (st) cudaStreamDestroy(st);
    return rc;
}

extern "C" int smat_zgemm(int mode, int m, int n, int k, const double *alpha, const double *A, int lda, const double *B,
                          int ldb, double *C, int ldc)
{
    using namespace smat::dense;
    if (m <= 0 || n <= 0 || k <= 0 || !alpha || !A || !B || !C || lda < m || ldb < k || ldc < m || (mode != 0 && mode != 1))
        return smat_fail(SMAT_EINVAL, "smat_zgemm: mode %d, m %d, n %d, k %d", mode, m, n, k);
    if (mode == 1 && !tc_available()) return smat_fail(SMAT_ECUDA, "smat_zgemm: the tensor-core product needs %s",
                                                       "more shared memory than this device gives a block");
    cudaStream_t st = nullptr;
    double2 *dA = nullptr, *dB = nullptr, *dC = nullptr;
    GemmCtx g{0, nullptr, 0, nullptr, 0, -1};
    int rc = SMAT_OK;
    const size_t an = (size_t)lda * k, bn = (size_t)ldb * n, cn = (size_t)ldc * n;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&dA, an * sizeof(double2)) != cudaSuccess || cudaMalloc(&dB, bn * sizeof(double2)) != cudaSuccess ||
        cudaMalloc(&dC, cn * sizeof(double2)) != cudaSuccess)
        rc = smat_fail(SMAT_ENOMEM, "smat_zgemm: device allocation");
    if (!rc && mode == 1) {
        g.ws_bytes = tc_workspace_bytes(m, n);
        if (cudaMalloc(&g.ws, g.ws_bytes) != cudaSuccess || cudaMalloc(&g.err, sizeof(int)) != cudaSuccess ||
            cudaMemsetAsync(g.err, 0, sizeof(int), st) != cudaSuccess)
            rc = smat_fail(SMAT_ENOMEM, "smat_zgemm: workspace");
        g.tc = 1;
    }
    if (!rc && (cudaMemcpyAsync(dA, A, an * sizeof(double2), cudaMemcpyHostToDevice, st) != cudaSuccess ||
                cudaMemcpyAsync(dB, B, bn * sizeof(double2), cudaMemcpyHostToDevice, st) != cudaSuccess ||
                cudaMemcpyAsync(dC, C, cn * sizeof(double2), cudaMemcpyHostToDevice, st) != cudaSuccess))
        rc = smat_fail(SMAT_ECUDA, "smat_zgemm: upload");
    if (!rc) rc = zgemm_acc(m, n, k, make_double2(alpha[0], alpha[1]), dA, lda, dB, ldb, dC, ldc, &g, st);
    if (!rc && (cudaMemcpyAsync(C, dC, cn * sizeof(double2), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = smat_fail(SMAT_ECUDA, "smat_zgemm: %s", cudaGetErrorString(cudaGetLastError()));
    if (!rc) rc = gemm_ctx_check(g);
    if (st) cudaStreamSynchronize(st);
    gemm_ctx_release(g);
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    if (st) cudaStreamDestroy(st);
    return rc;
}

namespace {
/* a seeded fill of n complex values in [-1, 1) (a hash of the index) */
__global__ void k_fill_z(double2 *p, long long n, unsigned seed)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long h = (unsigned long long)i * 0x9E3779B97F4A7C15ull + seed;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    p[i] = make_double2((double)(h & 0xFFFFFFFFull) / 2147483648.0 - 1.0, (double)(h >> 32) / 2147483648.0 - 1.0);
}
} // namespace

extern "C" int smat_zgemm_time(int mode, int m, int n, int k, int reps, double *ms)
{
    using namespace smat::dense;
    if (m <= 0 || n <= 0 || k <= 0 || reps <= 0 || !ms || (mode != 0 && mode != 1))
        return smat_fail(SMAT_EINVAL, "smat_zgemm_time: mode %d, m %d, n %d, k %d, reps %d", mode, m, n, k, reps);
    if (mode == 1 && !tc_available()) return smat_fail(SMAT_ECUDA, "smat_zgemm_time: no tensor-core form here");
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double2 *dA = nullptr, *dB = nullptr, *dC = nullptr;
    GemmCtx g{0, nullptr, 0, nullptr, 0, -1};
    int rc = SMAT_OK;
    const long long an = (long long)m * k, bn = (long long)k * n, cn = (long long)m * n;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess || cudaMalloc(&dA, an * sizeof(double2)) != cudaSuccess ||
        cudaMalloc(&dB, bn * sizeof(double2)) != cudaSuccess || cudaMalloc(&dC, cn * sizeof(double2)) != cudaSuccess)
        rc = smat_fail(SMAT_ENOMEM, "smat_zgemm_time: device allocation");
    if (!rc && mode == 1) {
        g.ws_bytes = tc_workspace_bytes(m, n);
        if (cudaMalloc(&g.ws, g.ws_bytes) != cudaSuccess || cudaMalloc(&g.err, sizeof(int)) != cudaSuccess ||
            cudaMemsetAsync(g.err, 0, sizeof(int), st) != cudaSuccess)
            rc = smat_fail(SMAT_ENOMEM, "smat_zgemm_time: workspace");
        g.tc = 1;
    }
    if (!rc) {
        k_fill_z<<<(unsigned)((an + 255) / 256), 256, 0, st>>>(dA, an, 1u);
        k_fill_z<<<(unsigned)((bn + 255) / 256), 256, 0, st>>>(dB, bn, 2u);
        k_fill_z<<<(unsigned)((cn + 255) / 256), 256, 0, st>>>(dC, cn, 3u);
        const double2 m1 = make_double2(-1.0, 0.0);
        rc = zgemm_acc(m, n, k, m1, dA, m, dB, k, dC, m, &g, st); /* warm-up */
        if (!rc && cudaEventRecord(e0, st) != cudaSuccess) rc = smat_fail(SMAT_ECUDA, "smat_zgemm_time: event");
        for (int r = 0; r < reps && !rc; r++) rc = zgemm_acc(m, n, k, m1, dA, m, dB, k, dC, m, &g, st);
        float t = 0.f;
        if (!rc && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                    cudaEventElapsedTime(&t, e0, e1) != cudaSuccess))
            rc = smat_fail(SMAT_ECUDA, "smat_zgemm_time: %s", cudaGetErrorString(cudaGetLastError()));
        if (!rc) rc = gemm_ctx_check(g);
        *ms = (double)t / reps;
    }
    if (st) cudaStreamSynchronize(st);
    gemm_ctx_release(g);
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    return rc;
}

extern "C" int smat_zgemm_wait_test(int *flag)
{
    using namespace smat::dense;
    if (!flag) return smat_fail(SMAT_EINVAL, "smat_zgemm_wait_test: null flag");
    if (!tc_available()) return smat_fail(SMAT_ECUDA, "smat_zgemm_wait_test: no tensor-core form here");
    const int m = 128, n = 32, k = 32;
    cudaStream_t st = nullptr;
    double2 *dA = nullptr, *dB = nullptr, *dC = nullptr;
    GemmCtx g{1, nullptr, 0, nullptr, 4096, 3};
    int rc = SMAT_OK;
    *flag = 0;
    g.ws_bytes = tc_workspace_bytes(m, n);
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&dA, sizeof(double2) * m * k) != cudaSuccess || cudaMalloc(&dB, sizeof(double2) * k * n) != cudaSuccess ||
        cudaMalloc(&dC, sizeof(double2) * m * n) != cudaSuccess || cudaMalloc(&g.ws, g.ws_bytes) != cudaSuccess ||
        cudaMalloc(&g.err, sizeof(int)) != cudaSuccess)
        rc = smat_fail(SMAT_ENOMEM, "smat_zgemm_wait_test: device allocation");
    if (!rc && (cudaMemsetAsync(dA, 0, sizeof(double2) * m * k, st) != cudaSuccess ||
                cudaMemsetAsync(dB, 0, sizeof(double2) * k * n, st) != cudaSuccess ||
                cudaMemsetAsync(dC, 0, sizeof(double2) * m * n, st) != cudaSuccess ||
                cudaMemsetAsync(g.err, 0, sizeof(int), st) != cudaSuccess))
        rc = smat_fail(SMAT_ECUDA, "smat_zgemm_wait_test: clear");
    if (!rc) rc = zgemm_acc_tc(m, n, k, make_double2(1.0, 0.0), dA, m, dB, k, dC, m, g, st);
    if (!rc && (cudaMemcpyAsync(flag, g.err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = smat_fail(SMAT_ECUDA, "smat_zgemm_wait_test: %s", cudaGetErrorString(cudaGetLastError()));
    if (st) cudaStreamSynchronize(st);
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    cudaFree(g.ws);
    cudaFree(g.err);
    if (st) cudaStreamDestroy(st);
    return rc;
}
