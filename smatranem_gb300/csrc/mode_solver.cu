/*
 * Port eigenmodes of one z layer on the GPU: the few-mode replacement for the
 * dense eigen solve of the reference mode solver (ModeCalc/Mcalc.c calc_Xi
 * :256-347; set_M :990-1066; dgeev_ / zgeev_ :858-861, :937-940).
 *
 * Mcalc forms two real symmetric matrices of order n = 2*L0*L1 from the
 * layer's media (set_V :1123, set_M :990; w = omega):
 *     maa = diag(w mu00, w mu11) + [Ddown1; -Ddown0] (1/(w eps22)) [Dup1, -Dup0]
 *     mbb = diag(w eps11, w eps00) + [Dup0; Dup1] (1/(w mu22)) [Ddown0, Ddown1]
 * with Dup the forward differences of set_D (:1088-1121, wrap factor BoundC at
 * the last column/row) and Ddown = -Dup^T, and then takes ALL eigenpairs of
 * mbb*maa densely: mbb*maa*H = (2 sin(theta/2))^2 H.  The propagating modes
 * -- the ones the FDTD excites and reports -- are the largest eigenvalues.
 * At a 256x192 cross-section n = 98,304 and the dense solve is out of reach.
 *
 * Here maa and mbb are stencils (never formed) and the leading eigenpairs
 * come from Chebyshev-filtered block subspace iteration:
 *   - the filter p(A) = T_d((A - c)/e) damps the interval [a, b] that holds
 *     the unwanted spectrum (a: below the spectral radius estimate, b: the
 *     smallest Ritz value of the block) and is fused into the two stencil
 *     kernels (three-term recurrence in the mbb kernel's epilogue);
 *   - Rayleigh-Ritz on an orthonormal basis of the filtered block, the small
 *     non-symmetric problem solved on the host by a complex Schur
 *     decomposition.  mbb*maa is self-adjoint only in the indefinite form
 *     x^T maa y: curl-rich evanescent directions carry a maa-norm about
 *     8/lambda times that of a propagating mode, so Rayleigh quotients in
 *     that form go far off for a block that is not yet clean; the Euclidean
 *     projection converges steadily (the large curl-curl and grad-div terms
 *     cancel in the product, C G = 0, so the operator is only mildly
 *     non-normal) and its converged Ritz pairs are eigenpairs to the
 *     residual tolerance.
 * The converged eigenvectors then go through Mcalc's own post-processing:
 * realizeH's gauge, makeSin, makeE, makeXi, normXi and degeneXi.
 *
 * Lossless media only: for a lossy layer the reference itself exits in
 * sortXi's final check (:620-626), so complex media are rejected here.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "host_internal.h"
#include "smatran_fdtd.h"
#include "trace.cuh"

namespace {

using cplx = std::complex<double>;

struct Op {
    int L0, L1, NA1;
    const double *V;  // 6*NA1: w mu00, w mu11, 1/(w eps22), w eps11, w eps00, 1/(w mu22) (FP64 copy)
    double s0, s1;    // diagonal of Dup0 / Dup1: -1, or BoundC when the axis has one cell
    double e0, e1;    // Dup's wrap coefficient at the last column / row (0 for a one-cell axis)
};

/* Y = maa X for the m columns of X (column j at X + j*ld).  One thread per
 * point p = i0 + L0*i1; w = (1/(w eps22)) (Dup1 x0 - Dup0 x1) is evaluated at
 * p and at its -e0 and -e1 neighbours, then
 *     y0 = V0 x0 + Ddown1 w,   y1 = V1 x1 - Ddown0 w,
 * with (Ddown_a w)(p) = -s_a w(p) - c_a(p - e_a) w(p - e_a). */
template <class T>
__global__ void k_maa(Op op, const T *__restrict__ Vt, const T *__restrict__ X, T *__restrict__ Y, long long ld)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= op.NA1) return;
    const int L0 = op.L0, L1 = op.L1, NA1 = op.NA1;
    const int i0 = p % L0, i1 = p / L0;
    const int i0m = i0 == 0 ? L0 - 1 : i0 - 1, i1m = i1 == 0 ? L1 - 1 : i1 - 1;
    const T s0 = (T)op.s0, s1 = (T)op.s1, e0 = (T)op.e0, e1 = (T)op.e1;
    const T *x0 = X + (long long)blockIdx.y * ld, *x1 = x0 + NA1;
    const T *V2 = Vt + 2 * (long long)NA1;
    auto cwt = [](int i, int La, T e) { return i < La - 1 ? (T)1 : e; };
    auto curl = [&](int j0, int j1) {  // w at (j0, j1)
        const int q = j0 + L0 * j1;
        const int q0 = (j0 + 1 == L0 ? 0 : j0 + 1) + L0 * j1, q1 = j0 + L0 * (j1 + 1 == L1 ? 0 : j1 + 1);
        const T d1 = s1 * __ldg(x0 + q) + cwt(j1, L1, e1) * __ldg(x0 + q1);
        const T d0 = s0 * __ldg(x1 + q) + cwt(j0, L0, e0) * __ldg(x1 + q0);
        return __ldg(V2 + q) * (d1 - d0);
    };
    const T wp = curl(i0, i1), wm0 = curl(i0m, i1), wm1 = curl(i0, i1m);
    T *y0 = Y + (long long)blockIdx.y * ld, *y1 = y0 + NA1;
    y0[p] = __ldg(Vt + p) * __ldg(x0 + p) + (-s1 * wp - cwt(i1m, L1, e1) * wm1);
    y1[p] = __ldg(Vt + NA1 + p) * __ldg(x1 + p) - (-s0 * wp - cwt(i0m, L0, e0) * wm0);
}

/* out = mbb W (W = maa Ycur), then Ynew = alpha*(out - c*Ycur) - beta*Yprev.
 *     u = (1/(w mu22)) (Ddown0 w0 + Ddown1 w1),
 *     out0 = V3 w0 + Dup0 u,   out1 = V4 w1 + Dup1 u.
 * alpha = 1, c = 0, beta = 0 gives the plain product A Ycur = mbb maa Ycur.
 * Ynew may alias Yprev (each thread reads its own entries before writing). */
template <class T>
__global__ void k_mbb(Op op, const T *__restrict__ Vt, const T *__restrict__ W, const T *Ycur, const T *Yprev, T *Ynew,
                      long long ld, T alpha, T c, T beta)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= op.NA1) return;
    const int L0 = op.L0, L1 = op.L1, NA1 = op.NA1;
    const int i0 = p % L0, i1 = p / L0;
    const T s0 = (T)op.s0, s1 = (T)op.s1, e0 = (T)op.e0, e1 = (T)op.e1;
    const long long col = (long long)blockIdx.y * ld;
    const T *w0 = W + col, *w1 = w0 + NA1;
    const T *V5 = Vt + 5 * (long long)NA1;
    auto cwt = [](int i, int La, T e) { return i < La - 1 ? (T)1 : e; };
    auto div = [&](int j0, int j1) {  // u at (j0, j1)
        const int q = j0 + L0 * j1;
        const int j0m = j0 == 0 ? L0 - 1 : j0 - 1, j1m = j1 == 0 ? L1 - 1 : j1 - 1;
        const T a0 = -s0 * __ldg(w0 + q) - cwt(j0m, L0, e0) * __ldg(w0 + j0m + L0 * j1);
        const T a1 = -s1 * __ldg(w1 + q) - cwt(j1m, L1, e1) * __ldg(w1 + j0 + L0 * j1m);
        return __ldg(V5 + q) * (a0 + a1);
    };
    const int i0p = i0 + 1 == L0 ? 0 : i0 + 1, i1p = i1 + 1 == L1 ? 0 : i1 + 1;
    const T up = div(i0, i1), up0 = div(i0p, i1), up1 = div(i0, i1p);
    const T o0 = __ldg(Vt + 3 * (long long)NA1 + p) * __ldg(w0 + p) + (s0 * up + cwt(i0, L0, e0) * up0);
    const T o1 = __ldg(Vt + 4 * (long long)NA1 + p) * __ldg(w1 + p) + (s1 * up + cwt(i1, L1, e1) * up1);
    const T *yc = Ycur + col;
    T r0 = alpha * (o0 - c * yc[p]), r1 = alpha * (o1 - c * yc[p + NA1]);
    if (beta != (T)0) {
        const T *yp = Yprev + col;
        r0 -= beta * yp[p];
        r1 -= beta * yp[p + NA1];
    }
    T *yn = Ynew + col;
    yn[p] = r0;
    yn[p + NA1] = r1;
}

/* The same operators in two passes each, every curl w (resp. divergence u)
 * evaluated once per point instead of at three points: half the FP64
 * operations (the stencils are FP64-pipe bound), the same expressions, so
 * the results are bit-identical to k_maa / k_mbb. */
template <class T>
__global__ void k_curl(Op op, const T *__restrict__ Vt, const T *__restrict__ X, T *__restrict__ Wc, long long ld)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= op.NA1) return;
    const int L0 = op.L0, L1 = op.L1, NA1 = op.NA1;
    const int j0 = p % L0, j1 = p / L0;
    const T s0 = (T)op.s0, s1 = (T)op.s1, e0 = (T)op.e0, e1 = (T)op.e1;
    const T *x0 = X + (long long)blockIdx.y * ld, *x1 = x0 + NA1;
    auto cwt = [](int i, int La, T e) { return i < La - 1 ? (T)1 : e; };
    const int q0 = (j0 + 1 == L0 ? 0 : j0 + 1) + L0 * j1, q1 = j0 + L0 * (j1 + 1 == L1 ? 0 : j1 + 1);
    const T d1 = s1 * __ldg(x0 + p) + cwt(j1, L1, e1) * __ldg(x0 + q1);
    const T d0 = s0 * __ldg(x1 + p) + cwt(j0, L0, e0) * __ldg(x1 + q0);
    Wc[(long long)blockIdx.y * ld + p] = __ldg(Vt + 2 * (long long)NA1 + p) * (d1 - d0);
}

template <class T>
__global__ void k_maa2(Op op, const T *__restrict__ Vt, const T *__restrict__ X, const T *__restrict__ Wc,
                       T *__restrict__ Y, long long ld)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= op.NA1) return;
    const int L0 = op.L0, L1 = op.L1, NA1 = op.NA1;
    const int i0 = p % L0, i1 = p / L0;
    const int i0m = i0 == 0 ? L0 - 1 : i0 - 1, i1m = i1 == 0 ? L1 - 1 : i1 - 1;
    const T s0 = (T)op.s0, s1 = (T)op.s1, e0 = (T)op.e0, e1 = (T)op.e1;
    auto cwt = [](int i, int La, T e) { return i < La - 1 ? (T)1 : e; };
    const long long col = (long long)blockIdx.y * ld;
    const T *x0 = X + col, *x1 = x0 + NA1, *w = Wc + col;
    const T wp = __ldg(w + p), wm0 = __ldg(w + i0m + L0 * i1), wm1 = __ldg(w + i0 + L0 * i1m);
    T *y0 = Y + col, *y1 = y0 + NA1;
    y0[p] = __ldg(Vt + p) * __ldg(x0 + p) + (-s1 * wp - cwt(i1m, L1, e1) * wm1);
    y1[p] = __ldg(Vt + NA1 + p) * __ldg(x1 + p) - (-s0 * wp - cwt(i0m, L0, e0) * wm0);
}

template <class T>
__global__ void k_div(Op op, const T *__restrict__ Vt, const T *__restrict__ W, T *__restrict__ U, long long ld)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= op.NA1) return;
    const int L0 = op.L0, L1 = op.L1, NA1 = op.NA1;
    const int j0 = p % L0, j1 = p / L0;
    const T s0 = (T)op.s0, s1 = (T)op.s1, e0 = (T)op.e0, e1 = (T)op.e1;
    auto cwt = [](int i, int La, T e) { return i < La - 1 ? (T)1 : e; };
    const T *w0 = W + (long long)blockIdx.y * ld, *w1 = w0 + NA1;
    const int j0m = j0 == 0 ? L0 - 1 : j0 - 1, j1m = j1 == 0 ? L1 - 1 : j1 - 1;
    const T a0 = -s0 * __ldg(w0 + p) - cwt(j0m, L0, e0) * __ldg(w0 + j0m + L0 * j1);
    const T a1 = -s1 * __ldg(w1 + p) - cwt(j1m, L1, e1) * __ldg(w1 + j0 + L0 * j1m);
    U[(long long)blockIdx.y * ld + p] = __ldg(Vt + 5 * (long long)NA1 + p) * (a0 + a1);
}

template <class T>
__global__ void k_mbb2(Op op, const T *__restrict__ Vt, const T *__restrict__ W, const T *__restrict__ Uc,
                       const T *Ycur, const T *Yprev, T *Ynew, long long ld, T alpha, T c, T beta)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= op.NA1) return;
    const int L0 = op.L0, L1 = op.L1, NA1 = op.NA1;
    const int i0 = p % L0, i1 = p / L0;
    const T s0 = (T)op.s0, s1 = (T)op.s1, e0 = (T)op.e0, e1 = (T)op.e1;
    auto cwt = [](int i, int La, T e) { return i < La - 1 ? (T)1 : e; };
    const long long col = (long long)blockIdx.y * ld;
    const T *w0 = W + col, *w1 = w0 + NA1, *u = Uc + col;
    const int i0p = i0 + 1 == L0 ? 0 : i0 + 1, i1p = i1 + 1 == L1 ? 0 : i1 + 1;
    const T up = __ldg(u + p), up0 = __ldg(u + i0p + L0 * i1), up1 = __ldg(u + i0 + L0 * i1p);
    const T o0 = __ldg(Vt + 3 * (long long)NA1 + p) * __ldg(w0 + p) + (s0 * up + cwt(i0, L0, e0) * up0);
    const T o1 = __ldg(Vt + 4 * (long long)NA1 + p) * __ldg(w1 + p) + (s1 * up + cwt(i1, L1, e1) * up1);
    const T *yc = Ycur + col;
    T r0 = alpha * (o0 - c * yc[p]), r1 = alpha * (o1 - c * yc[p + NA1]);
    if (beta != (T)0) {
        const T *yp = Yprev + col;
        r0 -= beta * yp[p];
        r1 -= beta * yp[p + NA1];
    }
    T *yn = Ynew + col;
    yn[p] = r0;
    yn[p + NA1] = r1;
}

/* column-major block conversion between FP64 and FP32 */
template <class A, class B>
__global__ void k_cvt(const A *__restrict__ in, B *__restrict__ out, long long count)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) out[t] = (B)in[t];
}

constexpr int GT = 256;       // threads of the reduction kernels
constexpr int GROWS = 32;     // rows staged per pass of k_gram
constexpr int MAXB = 128;     // largest block the kernels accept

/* partial Gram blocks: P[blk][i][j] = sum over this CTA's rows of X[r,i] Y[r,j] */
__global__ void k_gram(const double *__restrict__ X, const double *__restrict__ Y, long long n, long long ld, int mx,
                       int my, double *__restrict__ P)
{
    extern __shared__ double sm[];
    double *xs = sm, *ys = sm + GROWS * mx;
    const int nout = mx * my;
    const int per = (nout + GT - 1) / GT;  // <= MAXB*MAXB/GT = 64
    double acc[64];
    for (int k = 0; k < per; k++) acc[k] = 0.0;
    const long long chunk = (n + gridDim.x - 1) / gridDim.x;
    const long long r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
    for (long long rb = r0; rb < r1; rb += GROWS) {
        const int nr = (int)min((long long)GROWS, r1 - rb);
        __syncthreads();
        for (int t = threadIdx.x; t < GROWS * mx; t += GT) {
            const int r = t % GROWS, i = t / GROWS;
            xs[r + GROWS * i] = r < nr ? X[rb + r + ld * i] : 0.0;
        }
        for (int t = threadIdx.x; t < GROWS * my; t += GT) {
            const int r = t % GROWS, j = t / GROWS;
            ys[r + GROWS * j] = r < nr ? Y[rb + r + ld * j] : 0.0;
        }
        __syncthreads();
        for (int k = 0; k < per; k++) {
            const int o = threadIdx.x + GT * k;
            if (o >= nout) break;
            const int i = o % mx, j = o / mx;
            double s = acc[k];
            for (int r = 0; r < GROWS; r++) s = fma(xs[r + GROWS * i], ys[r + GROWS * j], s);
            acc[k] = s;
        }
    }
    for (int k = 0; k < per; k++) {
        const int o = threadIdx.x + GT * k;
        if (o < nout) P[(long long)blockIdx.x * nout + o] = acc[k];
    }
}

/* G[o] = sum over blocks of P[blk][o], blocks in order (deterministic) */
__global__ void k_sum_blocks(const double *__restrict__ P, int nblk, int nout, double *__restrict__ G)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nout) return;
    double s = 0.0;
    for (int b = 0; b < nblk; b++) s += P[(long long)b * nout + o];
    G[o] = s;
}

/* Y = X C: X is n x m (leading dimension ld), C is m x mo row-major in
 * (m x mo <= MAXB*MAXB doubles of) shared memory; thread = one row, 8 columns */
constexpr int GEMM_COLS = 8;
__global__ void k_gemm(const double *__restrict__ X, const double *__restrict__ Cm, long long n, long long ld, int m,
                       int mo, double *__restrict__ Y)
{
    extern __shared__ double cs[];
    for (int t = threadIdx.x; t < m * mo; t += blockDim.x) cs[t] = Cm[t];
    __syncthreads();
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int j0 = blockIdx.y * GEMM_COLS;
    if (r >= n) return;
    double acc[GEMM_COLS];
#pragma unroll
    for (int j = 0; j < GEMM_COLS; j++) acc[j] = 0.0;
    for (int k = 0; k < m; k++) {
        const double x = X[r + ld * k];
#pragma unroll
        for (int j = 0; j < GEMM_COLS; j++)
            if (j0 + j < mo) acc[j] = fma(x, cs[k * mo + j0 + j], acc[j]);
    }
#pragma unroll
    for (int j = 0; j < GEMM_COLS; j++)
        if (j0 + j < mo) Y[r + ld * (j0 + j)] = acc[j];
}

/* per column j: sum_r (A[r,j] - lam[j] B[r,j])^2 (lam == nullptr: sum A^2),
 * partial sums per CTA into P[blk][j] */
template <class T>
__global__ void k_colres(const T *__restrict__ A, const T *__restrict__ B, const double *__restrict__ lam,
                         long long n, long long ld, int m, double *__restrict__ P)
{
    __shared__ double red[GT];
    const long long chunk = (n + gridDim.x - 1) / gridDim.x;
    const long long r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
    for (int j = 0; j < m; j++) {
        const double l = lam ? lam[j] : 0.0;
        double s = 0.0;
        for (long long r = r0 + threadIdx.x; r < r1; r += GT) {
            const double v = lam ? (double)A[r + ld * j] - l * (double)B[r + ld * j] : (double)A[r + ld * j];
            s = fma(v, v, s);
        }
        red[threadIdx.x] = s;
        __syncthreads();
        for (int h = GT / 2; h > 0; h >>= 1) {
            if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x == 0) P[(long long)blockIdx.x * m + j] = red[0];
        __syncthreads();
    }
}

/* column j of A and of B scaled by s[j] (keeps the Chebyshev recurrence's
 * last two terms bounded; the recurrence is linear per column) */
template <class T>
__global__ void k_scale2(T *A, T *B, const double *__restrict__ s, long long n, long long ld, int m)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int j = 0; j < m; j++) {
        const T f = (T)s[j];
        A[r + ld * j] *= f;
        B[r + ld * j] *= f;
    }
}

/* deterministic uniform(-1, 1) fill (splitmix64 of seed and index) */
__global__ void k_random(double *X, long long n, long long ld, int j0, int m, unsigned long long seed)
{
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int j = j0; j < m; j++) {
        unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(r + n * j + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        X[r + ld * j] = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    }
}

/* ------------------------------------------------------------------ host */

#define MCK(call)                                                                                                      \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) {                                                                                       \
            rc = smat_fail(SMAT_ECUDA, "%s: %s", #call, cudaGetErrorString(e_));                                     \
            goto done;                                                                                                 \
        }                                                                                                              \
    } while (0)

/* Jacobi eigen-decomposition of the symmetric m x m matrix A (row-major,
 * destroyed): eigenvalues w (descending) and orthonormal eigenvectors as the
 * columns of V (row-major m x m).  Cyclic sweeps with the classical rotation
 * (Golub & Van Loan, Algorithm 8.5.3) until the off-diagonal part is below
 * 1e-15 of the Frobenius norm. */
void jacobi_eig(int m, std::vector<double> &A, std::vector<double> &w, std::vector<double> &V)
{
    V.assign((size_t)m * m, 0.0);
    for (int i = 0; i < m; i++) V[(size_t)i * m + i] = 1.0;
    double fro = 0.0;
    for (double a : A) fro += a * a;
    fro = std::sqrt(fro);
    for (int sweep = 0; sweep < 60 && fro > 0.0; sweep++) {
        double off = 0.0;
        for (int p = 0; p < m; p++)
            for (int q = p + 1; q < m; q++) off += 2.0 * A[(size_t)p * m + q] * A[(size_t)p * m + q];
        if (std::sqrt(off) <= 1e-15 * fro) break;
        for (int p = 0; p < m; p++)
            for (int q = p + 1; q < m; q++) {
                const double apq = A[(size_t)p * m + q];
                if (apq == 0.0) continue;
                const double app = A[(size_t)p * m + p], aqq = A[(size_t)q * m + q];
                const double tau = (aqq - app) / (2.0 * apq);
                const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
                for (int k = 0; k < m; k++) {  // A <- J^T A J
                    const double akp = A[(size_t)k * m + p], akq = A[(size_t)k * m + q];
                    A[(size_t)k * m + p] = c * akp - s * akq;
                    A[(size_t)k * m + q] = s * akp + c * akq;
                }
                for (int k = 0; k < m; k++) {
                    const double apk = A[(size_t)p * m + k], aqk = A[(size_t)q * m + k];
                    A[(size_t)p * m + k] = c * apk - s * aqk;
                    A[(size_t)q * m + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < m; k++) {
                    const double vkp = V[(size_t)k * m + p], vkq = V[(size_t)k * m + q];
                    V[(size_t)k * m + p] = c * vkp - s * vkq;
                    V[(size_t)k * m + q] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> ord(m);
    for (int i = 0; i < m; i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int a, int b) { return A[(size_t)a * m + a] > A[(size_t)b * m + b]; });
    std::vector<double> V2((size_t)m * m);
    w.resize(m);
    for (int j = 0; j < m; j++) {
        w[j] = A[(size_t)ord[j] * m + ord[j]];
        for (int k = 0; k < m; k++) V2[(size_t)k * m + j] = V[(size_t)k * m + ord[j]];
    }
    V.swap(V2);
}

/* Eigenvalues and eigenvectors of a general complex m x m matrix (row-major,
 * destroyed): Householder reduction to Hessenberg form, shifted QR with
 * Wilkinson shifts and Givens rotations to the complex Schur form
 * A = Z T Z^H (Golub & Van Loan, Algorithms 7.4.2 and 7.5.1 in complex
 * arithmetic), then the eigenvectors of T by back substitution, mapped by Z
 * and normalised to unit 2-norm.  Returns 0, or -1 if the QR iteration did
 * not converge. */
int small_eig(int m, std::vector<cplx> &A, std::vector<cplx> &w, std::vector<cplx> &Vout)
{
    auto at = [&](int i, int j) -> cplx & { return A[(size_t)i * m + j]; };
    std::vector<cplx> Zm((size_t)m * m, 0.0);
    auto z = [&](int i, int j) -> cplx & { return Zm[(size_t)i * m + j]; };
    for (int i = 0; i < m; i++) z(i, i) = 1.0;
    /* Hessenberg reduction */
    std::vector<cplx> v(m);
    for (int k = 0; k + 2 < m; k++) {
        double xn = 0.0;
        for (int i = k + 1; i < m; i++) xn += std::norm(at(i, k));
        xn = std::sqrt(xn);
        if (xn == 0.0) continue;
        const cplx x0 = at(k + 1, k);
        const cplx ph = std::abs(x0) > 0 ? x0 / std::abs(x0) : cplx(1.0, 0.0);
        for (int i = 0; i < m; i++) v[i] = 0.0;
        v[k + 1] = x0 + ph * xn;
        for (int i = k + 2; i < m; i++) v[i] = at(i, k);
        double vn = 0.0;
        for (int i = k + 1; i < m; i++) vn += std::norm(v[i]);
        if (vn == 0.0) continue;
        const double beta = 2.0 / vn;
        for (int j = 0; j < m; j++) {  // A <- (I - beta v v^H) A
            cplx s = 0.0;
            for (int i = k + 1; i < m; i++) s += std::conj(v[i]) * at(i, j);
            s *= beta;
            for (int i = k + 1; i < m; i++) at(i, j) -= v[i] * s;
        }
        for (int i = 0; i < m; i++) {  // A <- A (I - beta v v^H); Z likewise
            cplx s = 0.0, t = 0.0;
            for (int j = k + 1; j < m; j++) {
                s += at(i, j) * v[j];
                t += z(i, j) * v[j];
            }
            s *= beta;
            t *= beta;
            for (int j = k + 1; j < m; j++) {
                at(i, j) -= s * std::conj(v[j]);
                z(i, j) -= t * std::conj(v[j]);
            }
        }
        for (int i = k + 2; i < m; i++) at(i, k) = 0.0;
    }
    /* shifted QR on the Hessenberg matrix */
    const double eps = 2.220446049250313e-16;
    double anorm = 0.0;
    for (const cplx &a : A) anorm = std::max(anorm, std::abs(a));
    std::vector<double> gc(m);
    std::vector<cplx> gs(m);
    int hi = m - 1, iter = 0, total = 0;
    while (hi > 0) {
        int lo = hi;
        while (lo > 0) {
            const double sc = std::abs(at(lo - 1, lo - 1)) + std::abs(at(lo, lo));
            if (std::abs(at(lo, lo - 1)) <= eps * (sc > 0 ? sc : anorm)) {
                at(lo, lo - 1) = 0.0;
                break;
            }
            lo--;
        }
        if (lo == hi) {
            hi--;
            iter = 0;
            continue;
        }
        if (++total > 100 * m) return -1;
        cplx mu;
        if (iter > 0 && iter % 11 == 0) {  // exceptional shift
            mu = at(hi, hi) + std::abs(at(hi, hi - 1));
        } else {  // Wilkinson: eigenvalue of the trailing 2 x 2 closer to its last entry
            const cplx a = at(hi - 1, hi - 1), b = at(hi - 1, hi), c = at(hi, hi - 1), d = at(hi, hi);
            const cplx tr = a + d, det = a * d - b * c;
            const cplx disc = std::sqrt(tr * tr * 0.25 - det);
            const cplx l1 = tr * 0.5 + disc, l2 = tr * 0.5 - disc;
            mu = std::abs(l1 - d) < std::abs(l2 - d) ? l1 : l2;
        }
        iter++;
        for (int k = lo; k <= hi; k++) at(k, k) -= mu;
        for (int k = lo; k < hi; k++) {  // left rotations: zero the subdiagonal
            const cplx x = at(k, k), y = at(k + 1, k);
            const double r = std::sqrt(std::norm(x) + std::norm(y));
            double c;
            cplx sn;
            if (r == 0.0) {
                c = 1.0;
                sn = 0.0;
            } else {
                const double ax = std::abs(x);
                const cplx ux = ax > 0 ? x / ax : cplx(1.0, 0.0);
                c = ax / r;
                sn = ux * std::conj(y) / r;
            }
            gc[k] = c;
            gs[k] = sn;
            for (int j = k; j < m; j++) {  // [x'; y'] = [c, s; -conj(s), c] [x; y]
                const cplx p = at(k, j), q = at(k + 1, j);
                at(k, j) = c * p + sn * q;
                at(k + 1, j) = -std::conj(sn) * p + c * q;
            }
        }
        for (int k = lo; k < hi; k++) {  // right rotations (the adjoint), also on Z
            const double c = gc[k];
            const cplx sn = gs[k];
            const int rmax = std::min(k + 2, hi);
            for (int i = 0; i <= rmax; i++) {
                const cplx p = at(i, k), q = at(i, k + 1);
                at(i, k) = c * p + std::conj(sn) * q;
                at(i, k + 1) = -sn * p + c * q;
            }
            for (int i = 0; i < m; i++) {
                const cplx p = z(i, k), q = z(i, k + 1);
                z(i, k) = c * p + std::conj(sn) * q;
                z(i, k + 1) = -sn * p + c * q;
            }
        }
        for (int k = lo; k <= hi; k++) at(k, k) += mu;
    }
    /* eigenvectors of the triangular T, then x = Z y */
    w.resize(m);
    Vout.assign((size_t)m * m, 0.0);
    std::vector<cplx> y(m);
    const double small = eps * std::max(anorm, 1e-300);
    for (int k = 0; k < m; k++) {
        w[k] = at(k, k);
        for (int i = 0; i < m; i++) y[i] = 0.0;
        y[k] = 1.0;
        for (int i = k - 1; i >= 0; i--) {
            cplx s = 0.0;
            for (int j = i + 1; j <= k; j++) s += at(i, j) * y[j];
            cplx den = at(i, i) - at(k, k);
            if (std::abs(den) < small) den = small;
            y[i] = -s / den;
        }
        double nr = 0.0;
        std::vector<cplx> xv(m, 0.0);
        for (int i = 0; i < m; i++) {
            cplx s = 0.0;
            for (int j = 0; j <= k; j++) s += z(i, j) * y[j];
            xv[i] = s;
            nr += std::norm(s);
        }
        nr = std::sqrt(nr);
        for (int i = 0; i < m; i++) Vout[(size_t)i * m + k] = xv[i] / nr;
    }
    return 0;
}

template <class T> struct nd {
    using type = T;
};

struct Solver {
    Op op{};
    cudaStream_t st = nullptr;
    long long n = 0, ld = 0;
    int mb = 0, nblk = 0;
    double *dV = nullptr, *bufs[7] = {}, *dP = nullptr, *dG = nullptr, *dC = nullptr, *dL = nullptr;
    float *dVf = nullptr, *fbufs[4] = {};  /* FP32 copy of the coefficients; FP32 filter buffers */
    double *aux = nullptr;                 /* w or u of every point and column (two-pass stencils) */
    float *auxf = nullptr;
    long long matvecs = 0, matvecs32 = 0;

    ~Solver()
    {
        if (st) cudaStreamSynchronize(st);
        cudaFree(dV);
        cudaFree(dVf);
        for (double *b : bufs) cudaFree(b);
        for (float *b : fbufs) cudaFree(b);
        cudaFree(aux);
        cudaFree(auxf);
        cudaFree(dP);
        cudaFree(dG);
        cudaFree(dC);
        cudaFree(dL);
        if (st) cudaStreamDestroy(st);
    }
    dim3 pgrid(int m) const { return dim3((unsigned)((op.NA1 + 127) / 128), (unsigned)m); }

    const double *coef(const double *) const { return dV; }
    const float *coef(const float *) const { return dVf; }
    double *scratch(const double *) const { return aux; }
    float *scratch(const float *) const { return auxf; }
    bool two_pass = true;
    template <class T> int maa(const T *X, T *Y, int m)
    {
        if (two_pass) {
            T *w = scratch(X);
            k_curl<T><<<pgrid(m), 128, 0, st>>>(op, coef(X), X, w, ld);
            k_maa2<T><<<pgrid(m), 128, 0, st>>>(op, coef(X), X, w, Y, ld);
        } else {
            k_maa<T><<<pgrid(m), 128, 0, st>>>(op, coef(X), X, Y, ld);
        }
        return cudaPeekAtLastError() == cudaSuccess ? SMAT_OK : smat_fail(SMAT_ECUDA, "k_maa launch");
    }
    template <class T>
    int mbb(const T *W, const T *Yc, const typename nd<T>::type *Yp, T *Yn, int m, double alpha, double c, double beta)
    {
        if (two_pass) {
            T *u = scratch(W);
            k_div<T><<<pgrid(m), 128, 0, st>>>(op, coef(W), W, u, ld);
            k_mbb2<T><<<pgrid(m), 128, 0, st>>>(op, coef(W), W, u, Yc, Yp, Yn, ld, (T)alpha, (T)c, (T)beta);
        } else {
            k_mbb<T><<<pgrid(m), 128, 0, st>>>(op, coef(W), W, Yc, Yp, Yn, ld, (T)alpha, (T)c, (T)beta);
        }
        return cudaPeekAtLastError() == cudaSuccess ? SMAT_OK : smat_fail(SMAT_ECUDA, "k_mbb launch");
    }
    template <class A, class B> int convert(const A *in, B *out, int m)
    {
        const long long count = n * m;
        k_cvt<A, B><<<(unsigned)((count + 255) / 256), 256, 0, st>>>(in, out, count);
        return cudaPeekAtLastError() == cudaSuccess ? SMAT_OK : smat_fail(SMAT_ECUDA, "k_cvt launch");
    }
    /* G (host, mx x my row-major by i*my + j) = X^T Y */
    int gram(const double *X, const double *Y, int mx, int my, std::vector<double> &G)
    {
        const size_t smem = (size_t)GROWS * (mx + my) * sizeof(double);
        k_gram<<<nblk, GT, smem, st>>>(X, Y, n, ld, mx, my, dP);
        k_sum_blocks<<<(mx * my + 255) / 256, 256, 0, st>>>(dP, nblk, mx * my, dG);
        std::vector<double> g((size_t)mx * my);
        if (cudaMemcpyAsync(g.data(), dG, g.size() * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return smat_fail(SMAT_ECUDA, "gram: %s", cudaGetErrorString(cudaGetLastError()));
        G.assign((size_t)mx * my, 0.0);
        for (int j = 0; j < my; j++)
            for (int i = 0; i < mx; i++) G[(size_t)i * my + j] = g[i + (size_t)mx * j];
        return SMAT_OK;
    }
    /* Y = X C with C host row-major m x mo */
    int gemm(const double *X, const std::vector<double> &Cm, int m, int mo, double *Y)
    {
        if (cudaMemcpyAsync(dC, Cm.data(), (size_t)m * mo * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
            return smat_fail(SMAT_ECUDA, "gemm upload");
        const dim3 g((unsigned)((n + 127) / 128), (unsigned)((mo + GEMM_COLS - 1) / GEMM_COLS));
        k_gemm<<<g, 128, (size_t)m * mo * sizeof(double), st>>>(X, dC, n, ld, m, mo, Y);
        /* dC is reused by the next call: finish before returning */
        if (cudaStreamSynchronize(st) != cudaSuccess) return smat_fail(SMAT_ECUDA, "k_gemm");
        return SMAT_OK;
    }
    /* per column: ||A_j - lam_j B_j||^2 (lam empty: ||A_j||^2) */
    template <class T>
    int colres(const T *A, const typename nd<T>::type *B, const std::vector<double> &lam, int m,
               std::vector<double> &out)
    {
        if (!lam.empty() &&
            cudaMemcpyAsync(dL, lam.data(), (size_t)m * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
            return smat_fail(SMAT_ECUDA, "colres upload");
        k_colres<T><<<nblk, GT, 0, st>>>(A, B, lam.empty() ? nullptr : dL, n, ld, m, dP);
        k_sum_blocks<<<(m + 255) / 256, 256, 0, st>>>(dP, nblk, m, dG);
        out.resize(m);
        if (cudaMemcpyAsync(out.data(), dG, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return smat_fail(SMAT_ECUDA, "colres: %s", cudaGetErrorString(cudaGetLastError()));
        return SMAT_OK;
    }
    /* rescale columns of cur (and prev alike) to unit norm */
    template <class T> int rescale(T *cur, T *prev, int m)
    {
        std::vector<double> nv;
        int rc = colres<T>(cur, nullptr, {}, m, nv);
        if (rc) return rc;
        for (double &v : nv) v = (v > 0 && std::isfinite(v)) ? 1.0 / std::sqrt(v) : 1.0;
        if (cudaMemcpyAsync(dL, nv.data(), (size_t)m * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
            return smat_fail(SMAT_ECUDA, "rescale upload");
        k_scale2<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(cur, prev, dL, n, ld, m);
        if (cudaStreamSynchronize(st) != cudaSuccess) return smat_fail(SMAT_ECUDA, "k_scale2");
        return SMAT_OK;
    }
    void random(double *X, int j0, int m, unsigned long long seed)
    {
        if (j0 < m) k_random<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(X, n, ld, j0, m, seed);
    }
};

/* Chebyshev filter of degree d on [c - e, c + e], Y = T_d((A - c)/e) X0, in
 * the precision of T; Fa, Fb rotate with X0 (left untouched after the first
 * step), Wt holds maa Y_k; *out receives the buffer with the result */
template <class T>
int chebyshev(Solver &S, const T *X0, T *Fa, T *Fb, T *Wt, int mb, int degree, double c, double e, T **out)
{
    int rc;
    const T *prev = X0;
    T *cur = Fa;
    if ((rc = S.maa(prev, Wt, mb)) || (rc = S.mbb(Wt, prev, nullptr, cur, mb, 1.0 / e, c, 0.0))) return rc;
    for (int k = 1; k < degree; k++) {
        T *nxt = (prev == X0) ? Fb : const_cast<T *>(prev);
        if ((rc = S.maa(cur, Wt, mb)) || (rc = S.mbb(Wt, cur, prev, nxt, mb, 2.0 / e, c, 1.0))) return rc;
        prev = cur;
        cur = nxt;
        if (k % 32 == 0 && k + 1 < degree && (rc = S.rescale(cur, const_cast<T *>(prev), mb))) return rc;
    }
    *out = cur;
    return SMAT_OK;
}

int check_media(int L0, int L1, const int *bc, double omega, const double *med, std::vector<double> &V)
{
    if (L0 <= 0 || L1 <= 0 || (long long)L0 * L1 > (1LL << 28))
        return smat_fail(SMAT_EINVAL, "mode solver: bad lattice %d x %d", L0, L1);
    if (!bc || !med) return smat_fail(SMAT_EINVAL, "mode solver: null BoundC or media");
    for (int a = 0; a < 2; a++)
        if (bc[a] < -1 || bc[a] > 1) return smat_fail(SMAT_EINVAL, "mode solver: BoundC[%d] = %d", a, bc[a]);
    if (!(omega > 0.0) || !std::isfinite(omega)) return smat_fail(SMAT_EINVAL, "mode solver: omega = %g", omega);
    const long long NA1 = (long long)L0 * L1;
    V.resize(6 * NA1);
    for (long long k = 0; k < 6 * NA1; k++) {
        const double re = med[2 * k], im = med[2 * k + 1];
        if (im != 0.0)
            return smat_fail(SMAT_EINVAL,
                             "mode solver: complex port media (value %lld): the reference mode solver handles "
                             "lossless layers only (ModeCalc/Mcalc.c sortXi :620-626)", k);
        if (!std::isfinite(re) || re == 0.0) return smat_fail(SMAT_EINVAL, "mode solver: medium value %lld = %g", k, re);
        /* set_V :1150-1157: Vcomp = omega * med, rows 2 and 5 inverted */
        const double v = re * omega;
        const int row = (int)(k / NA1);
        V[k] = (row == 2 || row == 5) ? 1.0 / v : v;
    }
    return SMAT_OK;
}

int setup(Solver &S, int L0, int L1, const int *bc, const std::vector<double> &V, int mb)
{
    int rc = SMAT_OK;
    S.op.L0 = L0;
    S.op.L1 = L1;
    S.op.NA1 = L0 * L1;
    S.op.s0 = L0 > 1 ? -1.0 : (double)bc[0];
    S.op.s1 = L1 > 1 ? -1.0 : (double)bc[1];
    S.op.e0 = L0 > 1 ? (double)bc[0] : 0.0;
    S.op.e1 = L1 > 1 ? (double)bc[1] : 0.0;
    S.n = S.ld = 2LL * S.op.NA1;
    S.mb = mb;
    int dev = 0, sms = 148;
    MCK(cudaGetDevice(&dev));
    MCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    S.nblk = (int)std::min<long long>(2LL * sms, std::max<long long>(1, (S.n + 1023) / 1024));
    MCK(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
    MCK(cudaMalloc(&S.dV, V.size() * sizeof(double)));
    MCK(cudaMemcpyAsync(S.dV, V.data(), V.size() * sizeof(double), cudaMemcpyHostToDevice, S.st));
    S.op.V = S.dV;
    {   /* SMATRAN_MODE_ONE_PASS=1: the one-pass stencils (same results, for comparison) */
        const char *env = getenv("SMATRAN_MODE_ONE_PASS");
        S.two_pass = !(env && env[0] == '1');
    }
    for (double *&b : S.bufs) MCK(cudaMalloc(&b, (size_t)S.n * mb * sizeof(double)));
    for (float *&b : S.fbufs) MCK(cudaMalloc(&b, (size_t)S.n * mb * sizeof(float)));
    MCK(cudaMalloc(&S.aux, (size_t)S.n * mb * sizeof(double)));
    MCK(cudaMalloc(&S.auxf, (size_t)S.n * mb * sizeof(float)));
    MCK(cudaMalloc(&S.dVf, V.size() * sizeof(float)));
    {
        std::vector<float> vf(V.begin(), V.end());
        MCK(cudaMemcpyAsync(S.dVf, vf.data(), vf.size() * sizeof(float), cudaMemcpyHostToDevice, S.st));
        MCK(cudaStreamSynchronize(S.st));
    }
    MCK(cudaMalloc(&S.dP, (size_t)S.nblk * mb * mb * sizeof(double)));
    MCK(cudaMalloc(&S.dG, (size_t)mb * mb * sizeof(double)));
    MCK(cudaMalloc(&S.dC, (size_t)mb * mb * sizeof(double)));
    MCK(cudaMalloc(&S.dL, (size_t)mb * sizeof(double)));
    {
        int smem_optin = 0;
        MCK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        const int need = (int)std::max((size_t)GROWS * 2 * mb, (size_t)mb * mb) * (int)sizeof(double);
        if (need > smem_optin) { rc = smat_fail(SMAT_EINVAL, "mode solver: block of %d vectors too large", mb); goto done; }
        MCK(cudaFuncSetAttribute(k_gram, cudaFuncAttributeMaxDynamicSharedMemorySize, need));
        MCK(cudaFuncSetAttribute(k_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, need));
    }
done:
    return rc;
}

} // namespace

/* The host Schur solver of the Rayleigh-Ritz step, for testing: B is m x m
 * complex row-major (interleaved), w m complex, V m x m complex row-major
 * (eigenvector k in column k). */
extern "C" int smat_mode_small_eig(int m, const double *B, double *w, double *V)
{
    if (m <= 0 || m > 4096 || !B || !w || !V) return smat_fail(SMAT_EINVAL, "smat_mode_small_eig: m = %d", m);
    std::vector<cplx> A((const cplx *)B, (const cplx *)B + (size_t)m * m), ww, VV;
    if (small_eig(m, A, ww, VV)) return smat_fail(SMAT_ENUMERIC, "smat_mode_small_eig: QR did not converge");
    std::memcpy(w, ww.data(), sizeof(cplx) * m);
    std::memcpy(V, VV.data(), sizeof(cplx) * (size_t)m * m);
    return SMAT_OK;
}

extern "C" int smat_mode_apply(int L0, int L1, const int BoundC[2], double omega, const double *med, int which,
                               int m, const double *X, double *Y)
{
    std::vector<double> V;
    int rc = check_media(L0, L1, BoundC, omega, med, V);
    if (rc) return rc;
    if (which < 0 || which > 2 || m <= 0 || m > MAXB || !X || !Y)
        return smat_fail(SMAT_EINVAL, "smat_mode_apply: which = %d, m = %d", which, m);
    Solver S;
    if ((rc = setup(S, L0, L1, BoundC, V, m))) return rc;
    const size_t bytes = (size_t)S.n * m * sizeof(double);
    double *dX = S.bufs[0], *dW = S.bufs[1], *dZ = S.bufs[2];
    if (cudaMemcpyAsync(dX, X, bytes, cudaMemcpyHostToDevice, S.st) != cudaSuccess)
        return smat_fail(SMAT_ECUDA, "smat_mode_apply upload");
    double *out = dX;
    if (which == 0) {
        if ((rc = S.maa(dX, dW, m))) return rc;
        out = dW;
    } else if (which == 1) {
        if ((rc = S.mbb(dX, dX, nullptr, dZ, m, 1.0, 0.0, 0.0))) return rc;
        out = dZ;
    } else {
        if ((rc = S.maa(dX, dW, m)) || (rc = S.mbb(dW, dX, nullptr, dZ, m, 1.0, 0.0, 0.0))) return rc;
        out = dZ;
    }
    if (cudaMemcpyAsync(Y, out, bytes, cudaMemcpyDeviceToHost, S.st) != cudaSuccess ||
        cudaStreamSynchronize(S.st) != cudaSuccess)
        return smat_fail(SMAT_ECUDA, "smat_mode_apply: %s", cudaGetErrorString(cudaGetLastError()));
    return SMAT_OK;
}

extern "C" int smat_mode_solve(int L0, int L1, const int BoundC[2], double omega, const double *med, int nmodes,
                               const smat_mode_opts *opts, double *theta, double *Xi, smat_mode_info *info)
{
    smat::TraceRange trace_("smat_mode_solve");
    const auto t_start = std::chrono::steady_clock::now();
    std::vector<double> V;
    int rc = check_media(L0, L1, BoundC, omega, med, V);
    if (rc) return rc;
    const long long n = 2LL * L0 * L1;
    if (nmodes <= 0 || nmodes > n) return smat_fail(SMAT_EINVAL, "smat_mode_solve: nmodes = %d", nmodes);
    if (!theta || !Xi) return smat_fail(SMAT_EINVAL, "smat_mode_solve: null output");
    smat_mode_opts o{};
    if (opts) o = *opts;
    const double tol = o.tol > 0 ? o.tol : 1e-12;
    const int degree0 = o.degree > 0 ? o.degree : 24;
    const int max_iter = o.max_iter > 0 ? o.max_iter : 2000;
    int guard = o.guard > 0 ? o.guard : std::max(8, nmodes / 2);
    int mb = (int)std::min<long long>(n, (long long)nmodes + guard);
    if (mb > MAXB) return smat_fail(SMAT_EINVAL, "smat_mode_solve: %d modes + %d guard > %d", nmodes, guard, MAXB);
    const unsigned long long seed = o.seed ? o.seed : 0x5eed5eedull;

    Solver S;
    if ((rc = setup(S, L0, L1, BoundC, V, mb))) return rc;
    double *X = S.bufs[0], *AX = S.bufs[1], *W = S.bufs[2], *Z = S.bufs[3];
    double *F[3] = {S.bufs[4], S.bufs[5], S.bufs[6]};

    /* spectral radius by power iteration on one column */
    double rho = 0.0;
    {
        S.random(F[0], 0, 1, seed ^ 0xabcdefull);
        std::vector<double> nv;
        if ((rc = S.colres(F[0], nullptr, {}, 1, nv))) return rc;
        double nrm = std::sqrt(nv[0]);
        for (int it = 0; it < 80; it++) {
            if ((rc = S.maa(F[0], W, 1)) || (rc = S.mbb(W, F[0], nullptr, F[1], 1, 1.0 / nrm, 0.0, 0.0))) return rc;
            S.matvecs++;
            if ((rc = S.colres(F[1], nullptr, {}, 1, nv))) return rc;
            const double r = std::sqrt(nv[0]);  // ||A v|| / ||v||
            if (!std::isfinite(r)) return smat_fail(SMAT_ENUMERIC, "mode solver: non-finite operator norm");
            rho = std::max(rho, r);
            nrm = r;
            std::swap(F[0], F[1]);
        }
    }
    double a = -1.25 * rho, b = 0.0;
    S.random(X, 0, mb, seed);

    std::vector<double> lam, res, relres, Cm;
    double ltop = -INFINITY;  // largest Ritz value seen (estimate of the top eigenvalue)
    bool use32 = o.precision == 0;
    int iters = 0, found = 0, r = 0;
    bool done = false;
    for (iters = 1; iters <= max_iter && !done; iters++) {
        /* Chebyshev filter of degree d on [a, b]: Y = T_d((A - c)/e) X.  The
         * degree grows with the iteration count (up to 256): early passes
         * refresh the cut b often, late ones spend their time filtering the
         * slow modes at the edge of a dense (cladding) spectrum */
        const double c = 0.5 * (a + b), e = 0.5 * (b - a);
        int degree = std::min(256, degree0 * (1 + (iters - 1) / 4));
        /* ... but the top mode may outgrow the damped interval by at most
         * e^13 per pass, so that the block keeps its rank (the Gram
         * truncation below drops directions under 1e-13) */
        const double xt = (ltop - c) / e;
        if (std::isfinite(xt) && xt > 1.0) degree = std::min(degree, std::max(4, (int)(13.0 / std::acosh(xt))));
        /* FP32 passes while the wanted residuals are above 1e-6 (the filter
         * only shapes the subspace; GB300's FP32 rate is many times its FP64
         * rate), FP64 passes to finish; the Rayleigh-Ritz step is FP64 always */
        double *Y = nullptr;
        if (use32) {
            float *yf = nullptr;
            if ((rc = S.convert(X, S.fbufs[0], mb)) ||
                (rc = chebyshev<float>(S, S.fbufs[0], S.fbufs[1], S.fbufs[2], S.fbufs[3], mb, degree, c, e, &yf)) ||
                (rc = S.convert(yf, F[0], mb)))
                return rc;
            Y = F[0];
            S.matvecs32 += (long long)degree * mb;
        } else {
            if ((rc = chebyshev<double>(S, X, F[0], F[1], W, mb, degree, c, e, &Y))) return rc;
            S.matvecs += (long long)degree * mb;
        }
        /* Rayleigh-Ritz on an orthonormal basis of the filtered block:
         * Q = Y T (T from the Gram matrix's eigen-decomposition, directions
         * below 1e-13 of the largest dropped), B = Q^T A Q, Ritz pairs from
         * the small non-symmetric eigenproblem */
        if ((rc = S.maa(Y, W, mb)) || (rc = S.mbb(W, Y, nullptr, Z, mb, 1.0, 0.0, 0.0))) return rc;
        S.matvecs += mb;
        std::vector<double> G, Fm;
        if ((rc = S.gram(Y, Y, mb, mb, G)) || (rc = S.gram(Y, Z, mb, mb, Fm))) return rc;
        std::vector<double> d(mb);
        for (int i = 0; i < mb; i++) d[i] = G[(size_t)i * mb + i] > 0 ? 1.0 / std::sqrt(G[(size_t)i * mb + i]) : 0.0;
        for (int i = 0; i < mb; i++)
            for (int j = i; j < mb; j++) {
                const double gij = 0.5 * (G[(size_t)i * mb + j] + G[(size_t)j * mb + i]) * d[i] * d[j];
                G[(size_t)i * mb + j] = G[(size_t)j * mb + i] = gij;
            }
        std::vector<double> g, P;
        jacobi_eig(mb, G, g, P);
        r = 0;
        while (r < mb && g[r] > 1e-13 * g[0]) r++;
        if (r == 0) return smat_fail(SMAT_ENUMERIC, "mode solver: the filtered block vanished");
        std::vector<double> T((size_t)mb * r);  // T = D P g^{-1/2}
        for (int i = 0; i < mb; i++)
            for (int j = 0; j < r; j++) T[(size_t)i * r + j] = d[i] * P[(size_t)i * mb + j] / std::sqrt(g[j]);
        std::vector<double> FT((size_t)mb * r);
        for (int i = 0; i < mb; i++)
            for (int j = 0; j < r; j++) {
                double acc = 0.0;
                for (int q = 0; q < mb; q++) acc += Fm[(size_t)i * mb + q] * T[(size_t)q * r + j];
                FT[(size_t)i * r + j] = acc;
            }
        std::vector<cplx> B((size_t)r * r), w, U;
        for (int i = 0; i < r; i++)
            for (int j = 0; j < r; j++) {
                double acc = 0.0;
                for (int q = 0; q < mb; q++) acc += T[(size_t)q * r + i] * FT[(size_t)q * r + j];
                B[(size_t)i * r + j] = acc;
            }
        if (small_eig(r, B, w, U)) return smat_fail(SMAT_ENUMERIC, "mode solver: Rayleigh-Ritz QR did not converge");
        std::vector<int> ord(r);
        for (int i = 0; i < r; i++) ord[i] = i;
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return w[x].real() > w[y].real(); });
        /* a real basis of the Ritz vectors: a real eigenvalue's vector rotated
         * real; a complex pair (unconverged) kept as its real and imaginary parts */
        std::vector<double> Cr((size_t)r * r, 0.0);
        std::vector<char> is_c(r, 0);
        lam.assign(r, 0.0);
        for (int j = 0; j < r;) {
            const int o = ord[j];
            const cplx wj = w[o];
            if (std::fabs(wj.imag()) <= 1e-12 * std::max(1.0, std::fabs(wj.real()))) {
                int imx = 0;
                for (int i = 1; i < r; i++)
                    if (std::abs(U[(size_t)i * r + o]) > std::abs(U[(size_t)imx * r + o])) imx = i;
                const cplx u = U[(size_t)imx * r + o];
                const cplx ph = std::conj(u) / std::abs(u);
                double nr = 0.0;
                for (int i = 0; i < r; i++) nr += std::pow((U[(size_t)i * r + o] * ph).real(), 2);
                nr = std::sqrt(nr);
                for (int i = 0; i < r; i++) Cr[(size_t)i * r + j] = (U[(size_t)i * r + o] * ph).real() / nr;
                lam[j] = wj.real();
                j++;
            } else {
                for (int i = 0; i < r; i++) Cr[(size_t)i * r + j] = U[(size_t)i * r + o].real();
                lam[j] = wj.real();
                is_c[j] = 1;
                if (j + 1 < r) {
                    for (int i = 0; i < r; i++) Cr[(size_t)i * r + j + 1] = U[(size_t)i * r + o].imag();
                    lam[j + 1] = wj.real();
                    is_c[j + 1] = 1;
                }
                j += 2;
            }
        }
        Cm.assign((size_t)mb * r, 0.0);  // C = T Cr
        for (int i = 0; i < mb; i++)
            for (int j = 0; j < r; j++) {
                double acc = 0.0;
                for (int q = 0; q < r; q++) acc += T[(size_t)i * r + q] * Cr[(size_t)q * r + j];
                Cm[(size_t)i * r + j] = acc;
            }
        if ((rc = S.gemm(Y, Cm, mb, r, X)) || (rc = S.gemm(Z, Cm, mb, r, AX))) return rc;
        /* residuals relative to the spectral radius */
        std::vector<double> xn;
        if ((rc = S.colres(AX, X, lam, r, res)) || (rc = S.colres(X, nullptr, {}, r, xn))) return rc;
        relres.resize(r);
        for (int j = 0; j < r; j++)
            relres[j] = is_c[j] ? INFINITY : std::sqrt(res[j]) / (rho * std::sqrt(xn[j]));
        found = 0;
        while (found < r && found < nmodes && lam[found] > 0.0 && relres[found] <= tol) found++;
        if (use32) {
            double worst = 0.0;
            for (int j = 0; j < std::min(nmodes, r); j++)
                if (lam[j] > 0.0) worst = std::max(worst, relres[j]);
            if (worst <= 1e-6) use32 = false;
        }
        /* stop: all wanted found, or the next Ritz pair is a converged
         * non-propagating one (the layer has no more propagating modes) */
        if (found >= nmodes || (found < r && lam[found] <= 0.0 && relres[found] <= tol && iters > 3)) done = true;
        /* next interval: damp everything below the block's smallest Ritz
         * value (kept while the block has too few Ritz values to place it) */
        ltop = std::max(ltop, lam[0]);
        if (lam[r - 1] < a) a = lam[r - 1] - 0.25 * std::fabs(lam[r - 1]);
        if (r >= std::min(mb, nmodes + 2)) b = std::max(lam[r - 1], a + 1e-3 * (lam[0] - a));
        if (r < mb) S.random(X, r, mb, seed + 7919ull * iters);
    }
    if (found == 0) return smat_fail(SMAT_ENUMERIC, "mode solver: no propagating mode converged (%d iterations)", iters - 1);

    /* post-processing on the found modes, in Mcalc's steps; forward column j
     * of Xi at j, backward at K + j (K = nmodes), unfound columns zero */
    const int k = found, K = nmodes;
    std::vector<double> H((size_t)n * k), E((size_t)n * k);
    if ((rc = S.maa(X, W, k))) return rc;
    if (cudaMemcpyAsync(H.data(), X, H.size() * sizeof(double), cudaMemcpyDeviceToHost, S.st) != cudaSuccess ||
        cudaMemcpyAsync(E.data(), W, E.size() * sizeof(double), cudaMemcpyDeviceToHost, S.st) != cudaSuccess ||
        cudaStreamSynchronize(S.st) != cudaSuccess)
        return smat_fail(SMAT_ECUDA, "mode solver download: %s", cudaGetErrorString(cudaGetLastError()));
    const long long N2 = 2 * n;  // rows of Xi
    cplx *Xc = reinterpret_cast<cplx *>(Xi);
    cplx *th = reinterpret_cast<cplx *>(theta);
    std::memset(Xi, 0, sizeof(cplx) * (size_t)N2 * 2 * K);
    std::memset(theta, 0, sizeof(cplx) * 2 * (size_t)K);
    double max_res = 0.0;
    for (int j = 0; j < k; j++) {
        double *h = &H[(size_t)n * j], *ev = &E[(size_t)n * j];
        /* gauge: largest |H| entry positive (dgeev leaves the sign open) */
        long long imax = 0;
        for (long long i = 1; i < n; i++)
            if (std::fabs(h[i]) > std::fabs(h[imax])) imax = i;
        const double sg = h[imax] < 0 ? -1.0 : 1.0;
        /* makeSin :821-831 and makeE :731-757: E = maa H * conj(s)/|s|^2 */
        const double s = std::sqrt(lam[j]);
        const double f = s / (s * s);
        /* makeXi :645-666 */
        const cplx t = 2.0 * std::asin(cplx(0.5 * s, 0.0));
        th[j] = t;
        th[j + K] = -t;
        const cplx pm = std::exp(cplx(0.0, -0.5) * t), pp = std::exp(cplx(0.0, 0.5) * t);
        cplx *fw = Xc + N2 * j, *bw = Xc + N2 * (j + K);
        for (long long i = 0; i < n; i++) {
            const double hv = sg * h[i], evv = sg * ev[i] * f;
            fw[i] = pm * hv;
            bw[i] = pp * hv;
            fw[i + n] = cplx(evv, 0.0);
            bw[i + n] = cplx(-evv, 0.0);
        }
        max_res = std::max(max_res, relres[j]);
    }
    /* normXi :529-561, real-mode branch */
    auto norm_col = [&](int j) -> int {
        for (int fb = 0; fb < 2; fb++) {
            cplx *col = Xc + N2 * (j + fb * K);
            cplx z = 0.0;
            for (long long i = 0; i < n; i++) {
                z += std::conj(col[i]) * col[i + n];
                z += std::conj(col[i + n]) * col[i];
            }
            if ((0.5 - fb) * z.real() < 0.0)
                return smat_fail(SMAT_ENUMERIC, "flow direction error in normXi at mode %d (fb = %d)", j, fb);
            const double nr = 1.0 / std::sqrt(std::fabs(z.real()));
            for (long long i = 0; i < N2; i++) col[i] *= nr;
        }
        return SMAT_OK;
    };
    for (int j = 0; j < k; j++)
        if ((rc = norm_col(j))) return rc;
    /* degeneXi :417-467 among the returned modes; the dual columns are makePsi's
     * (:505-527) real-mode form: Psi_j = [E_j; H_j], Psi_{j+k} = -[E_{j+k}; H_{j+k}] */
    auto psi_dot = [&](int pcol, int xcol, double sign) {
        const cplx *P = Xc + N2 * pcol, *Xv = Xc + N2 * xcol;
        cplx z = 0.0;
        for (long long i = 0; i < n; i++) z += std::conj(sign * P[i + n]) * Xv[i];
        for (long long i = 0; i < n; i++) z += std::conj(sign * P[i]) * Xv[i + n];
        return z;
    };
    int ndegen = 0;
    const double FLT_EPS = 1.1920928955078125e-07;
    for (int j = 0; j < k - 1; j++)
        for (int i = j + 1; i < k; i++) {
            if (std::abs((th[j] - th[i]) / (th[j] + th[i])) >= FLT_EPS) continue;
            const cplx s_ij0 = psi_dot(i, j, 1.0), s_ijN = psi_dot(i + K, j + K, -1.0);
            const cplx s_ji0 = psi_dot(j, i, 1.0), s_jiN = psi_dot(j + K, i + K, -1.0);
            const double a0 = 1.0 / std::sqrt(std::abs(1.0 - s_ji0 * s_ij0));
            const double aN = 1.0 / std::sqrt(std::abs(1.0 - s_jiN * s_ijN));
            const cplx b0 = -a0 * s_ji0, bN = -aN * s_jiN;
            cplx *ci = Xc + N2 * i, *cj = Xc + N2 * j, *ciN = Xc + N2 * (i + K), *cjN = Xc + N2 * (j + K);
            for (long long q = 0; q < N2; q++) {
                ci[q] = a0 * ci[q] + b0 * cj[q];
                ciN[q] = aN * ciN[q] + bN * cjN[q];
            }
            if ((rc = norm_col(i))) return rc;
            ndegen++;
        }
    if (info) {
        info->n_found = k;
        info->iterations = iters - 1;
        info->matvecs = S.matvecs + S.matvecs32;
        info->matvecs_fp32 = S.matvecs32;
        info->max_residual = max_res;
        info->spectral_radius = rho;
        info->degenerate_pairs = ndegen;
        info->block = mb;
        info->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    }
    return SMAT_OK;
}
