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
              int ldc, cudaStream_t st)
{
    if (m <= 0 || n <= 0 || k <= 0) return SMAT_OK;
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

/* row interchanges ipiv[k0..k1) (absolute rows) applied in order to the
 * columns [c0, c1) of A; one thread per column */
__global__ void k_laswp(double2 *A, int lda, int c0, int c1, const int *__restrict__ ipiv, int k0, int k1)
{
    const int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    double2 *col = A + (long long)lda * c;
    for (int k = k0; k < k1; k++) {
        const int p = ipiv[k];
        if (p != k) {
            const double2 t = col[k];
            col[k] = col[p];
            col[p] = t;
        }
    }
}

/* X (nb x ncols at X, leading dimension ldx) <- T^{-1} X with T the nb x nb
 * triangle at T (unit lower if lower, else non-unit upper); one thread per
 * column, the triangle staged in shared memory */
constexpr int NBMAX = 32;
__global__ void k_trsm(const double2 *__restrict__ T, int ldt, int nb, double2 *X, int ldx, int ncols, int lower)
{
    __shared__ double2 ts[NBMAX][NBMAX + 1];
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
        const int r = t % nb, c = t / nb;
        ts[r][c] = T[r + (long long)ldt * c];
    }
    __syncthreads();
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= ncols) return;
    double2 x[NBMAX];
    double2 *xc = X + (long long)ldx * col;
    for (int r = 0; r < nb; r++) x[r] = xc[r];
    if (lower) {
        for (int r = 0; r < nb; r++) {
            double2 s = x[r];
            for (int k = 0; k < r; k++) s = cfms(s, ts[r][k], x[k]);
            x[r] = s;
        }
    } else {
        for (int r = nb - 1; r >= 0; r--) {
            double2 s = x[r];
            for (int k = r + 1; k < nb; k++) s = cfms(s, ts[r][k], x[k]);
            x[r] = cmul(s, crecip(ts[r][r]));
        }
    }
    for (int r = 0; r < nb; r++) xc[r] = x[r];
}

static int launch_ok(const char *what)
{
    return cudaPeekAtLastError() == cudaSuccess ? SMAT_OK : smat_fail(SMAT_ECUDA, "%s launch", what);
}

int getrf(int n, double2 *A, int lda, int *ipiv, int *info, cudaStream_t st)
{
    const double2 m1 = make_double2(-1.0, 0.0);
    for (int j = 0; j < n; j += NBMAX) {
        const int nb = std::min(NBMAX, n - j);
        k_panel<<<1, PT, 0, st>>>(A + j + (long long)lda * j, lda, n - j, nb, j, ipiv + j, info);
        if (int rc = launch_ok("k_panel")) return rc;
        /* the panel's pivots are local to rows [j, n): make them absolute is done
         * in k_panel (row0 = j); apply them left and right of the panel */
        if (j > 0) {
            k_laswp<<<(j + 127) / 128, 128, 0, st>>>(A, lda, 0, j, ipiv, j, j + nb);
            if (int rc = launch_ok("k_laswp")) return rc;
        }
        const int right = n - j - nb;
        if (right > 0) {
            k_laswp<<<(right + 127) / 128, 128, 0, st>>>(A, lda, j + nb, n, ipiv, j, j + nb);
            if (int rc = launch_ok("k_laswp")) return rc;
            k_trsm<<<(right + 127) / 128, 128, 0, st>>>(A + j + (long long)lda * j, lda, nb,
                                                         A + j + (long long)lda * (j + nb), lda, right, 1);
            if (int rc = launch_ok("k_trsm")) return rc;
            if (int rc = zgemm_acc(n - j - nb, right, nb, m1, A + (j + nb) + (long long)lda * j, lda,
                                   A + j + (long long)lda * (j + nb), lda, A + (j + nb) + (long long)lda * (j + nb),
                                   lda, st))
                return rc;
        }
    }
    return SMAT_OK;
}

int getrs(int n, int nrhs, const double2 *LU, int lda, const int *ipiv, double2 *B, int ldb, cudaStream_t st)
{
    if (n <= 0 || nrhs <= 0) return SMAT_OK;
    const double2 m1 = make_double2(-1.0, 0.0);
    k_laswp<<<(nrhs + 127) / 128, 128, 0, st>>>(B, ldb, 0, nrhs, ipiv, 0, n);
    if (int rc = launch_ok("k_laswp")) return rc;
    for (int j = 0; j < n; j += NBMAX) {  // L y = b
        const int nb = std::min(NBMAX, n - j);
        k_trsm<<<(nrhs + 127) / 128, 128, 0, st>>>(LU + j + (long long)lda * j, lda, nb, B + j, ldb, nrhs, 1);
        if (int rc = launch_ok("k_trsm")) return rc;
        if (int rc = zgemm_acc(n - j - nb, nrhs, nb, m1, LU + (j + nb) + (long long)lda * j, lda, B + j, ldb,
                               B + j + nb, ldb, st))
            return rc;
    }
    for (int j = ((n - 1) / NBMAX) * NBMAX; j >= 0; j -= NBMAX) {  // U x = y
        const int nb = std::min(NBMAX, n - j);
        k_trsm<<<(nrhs + 127) / 128, 128, 0, st>>>(LU + j + (long long)lda * j, lda, nb, B + j, ldb, nrhs, 0);
        if (int rc = launch_ok("k_trsm")) return rc;
        if (int rc = zgemm_acc(j, nrhs, nb, m1, LU + (long long)lda * j, lda, B + j, ldb, B, ldb, st)) return rc;
    }
    return SMAT_OK;
}

} // namespace dense
} // namespace smat

/* ---- test hook ------------------------------------------------------------ */

extern "C" int smat_zgesv(int n, int nrhs, const double *A, const double *B, double *X, int *info_out)
{
    using namespace smat::dense;
    if (n <= 0 || nrhs <= 0 || !A || !B || !X) return smat_fail(SMAT_EINVAL, "smat_zgesv: n = %d, nrhs = %d", n, nrhs);
    cudaStream_t st = nullptr;
    double2 *dA = nullptr, *dB = nullptr;
    int *dp = nullptr, *dinfo = nullptr;
    int rc = SMAT_OK, info = 0;
    const size_t an = (size_t)n * n, bn = (size_t)n * nrhs;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&dA, an * sizeof(double2)) != cudaSuccess || cudaMalloc(&dB, bn * sizeof(double2)) != cudaSuccess ||
        cudaMalloc(&dp, (size_t)n * sizeof(int)) != cudaSuccess || cudaMalloc(&dinfo, sizeof(int)) != cudaSuccess)
        rc = smat_fail(SMAT_ENOMEM, "smat_zgesv: device allocation");
    if (!rc && (cudaMemcpyAsync(dA, A, an * sizeof(double2), cudaMemcpyHostToDevice, st) != cudaSuccess ||
                cudaMemcpyAsync(dB, B, bn * sizeof(double2), cudaMemcpyHostToDevice, st) != cudaSuccess ||
                cudaMemsetAsync(dinfo, 0, sizeof(int), st) != cudaSuccess))
        rc = smat_fail(SMAT_ECUDA, "smat_zgesv: upload");
    if (!rc) rc = getrf(n, dA, n, dp, dinfo, st);
    if (!rc) rc = getrs(n, nrhs, dA, n, dp, dB, n, st);
    if (!rc && (cudaMemcpyAsync(X, dB, bn * sizeof(double2), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = smat_fail(SMAT_ECUDA, "smat_zgesv: %s", cudaGetErrorString(cudaGetLastError()));
    if (info_out) *info_out = info;
    if (st) cudaStreamSynchronize(st);
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dp);
    cudaFree(dinfo);
    if (st) cudaStreamDestroy(st);
    return rc;
}
