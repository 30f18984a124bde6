/*
 * FP64-accurate complex multiply-add on the tensor cores: C += alpha * A * B
 * with A (m x k), B (k x n), C (m x n) complex FP64, column-major -- the
 * zgemm_ of the layer transfer (Smat/Scalc.c inv_process :316-400 through the
 * blocked LU of dense_z.cu), computed by the Ozaki scheme (Ozaki, Ogita,
 * Oishi, Rump, "Error-free transformations of matrix multiplication by using
 * fast routines of matrix multiplication and its applications", Numer.
 * Algorithms 59, 2012), in the tensor-core form of Mukunoki, Ozaki, Ogita and
 * Imamura ("DGEMM using Tensor Cores, and Its Accurate and Reproducible
 * Versions", ISC 2020): every operand is cut into S slices of small integers
 * that the bf16 tensor cores multiply and an FP32 accumulator sums exactly.
 *
 *   - complex as real: [Pr | Pi] = [Ar | Ai] * [[Br, Bi], [-Bi, Br]], one real
 *     product of inner size 2k.
 *   - each row r of [Ar | Ai] is scaled by 2^-e_r (e_r: the exponent of its
 *     largest entry, so every scaled entry x lies in (-1, 1)) and cut into
 *     balanced base-256 digits of F = rint(x 2^55): x ~ sum_i t_i 2^(-7-8i),
 *     t_i integers in [-128, 128], exact in bf16; each column of the real B
 *     likewise (one exponent per complex column).
 *   - products t * t' are at most 2^14 in magnitude; with 2k <= 64 and at most
 *     S pairs per sum, every partial sum is an integer below 2^24 and the FP32
 *     accumulation of the tensor cores is exact.  The pairs (i, l) with the
 *     same i + l = d share the scale 2^(-14-8d) and one TMEM accumulator.
 *   - the d-accumulators are combined exactly in integers, X = sum_d acc_d
 *     256^(S-1-d), rounded once to the nearest double, scaled by
 *     2^(e_r + e_c - 14 - 8(S-1)) (exact), multiplied by alpha and added to C.
 *   Error: the cuts keep 55 bits below each row's (column's) leading bit and
 *   the pairs with i + l >= S are dropped, about 2k * S * 2^(-8S) of |row
 *   max| * |col max| per entry: 2^-47 relative for S = 7 at 2k = 64, the size
 *   of the FP64 product's own rounding bound over that inner size.
 *
 * GB300 form.  Output tiles of 128 rows x 16 complex columns, two CTAs of
 * 256 threads per SM (224 TMEM columns each), so that one CTA's epilogue runs
 * beside the other's products.  The slices are written by the two cutting
 * kernels (integer digit extraction: one FP64 multiply and one conversion per
 * value) as images of the shared-memory operand tiles (K-major, no swizzle:
 * core matrices of 8 rows x 16 bytes), so one thread loads them with bulk
 * async copies (cp.async.bulk, completion on mbarriers: every B slice at
 * once, the A slices through a ring of three buffers) and issues the
 * tcgen05.mma (kind::f16, bf16 x bf16 -> f32, M = 128, N = 32, K = 16) of
 * slice i as soon as it has landed; the S accumulators (32 TMEM columns each)
 * are read back by all eight warps (tcgen05.ld, one row per thread) for an
 * integer epilogue (exact int64 sum of the digit levels, the double assembled
 * from its bits) with one FP64 multiply-add per output: GB300's FP64 pipe
 * runs a few operations per clock per SM, so FP64 arithmetic is kept off every
 * per-element path.  Inner sizes above 32 are cut into passes of 32 complex
 * terms, each adding into C.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "dense_z.cuh"
#include "host_internal.h"
#include "smatran_fdtd.h"

namespace smat {
namespace dense {
namespace {

constexpr int S = 7;                 /* slices per operand */
constexpr int BM = 128;              /* tile rows (TMEM lanes) */
constexpr int BNC = 16;              /* complex columns per tile */
constexpr int BN = 2 * BNC;          /* real MMA columns: Pr then Pi */
constexpr int KI = 64;               /* bf16 inner size of an image: [re (32) | im (32)] */
constexpr int KC = KI / 2;           /* complex inner terms per pass */
constexpr int AIMG = BM * KI * 2;    /* bytes of an A slice image (16 KB) */
constexpr int BIMG = BN * KI * 2;    /* bytes of a B slice image (4 KB) */
constexpr int RING = 3;              /* A slice buffers */
constexpr int TMEM_COLS = 256;       /* S * BN = 224 columns used: two CTAs per SM fit TMEM */
constexpr int SMEM = RING * AIMG + S * BIMG + 8 * (2 * RING + 2) + 16;
constexpr unsigned WAIT_LIMIT = 1u << 24;

static_assert(S * BN <= TMEM_COLS, "accumulators exceed the TMEM allocation");
static_assert(S * KI * 128 * 128 < (1 << 24), "partial sums must stay exact in FP32");

/* byte offset of element (row, kk) in an operand image: 8-row groups of 1024
 * bytes, each holding the 8 core matrices (8 rows x 8 bf16) of the inner
 * dimension in order; so the inner-direction core-matrix stride (LBO) is 128
 * bytes and the 8-row-group stride (SBO) 1024 */
__host__ __device__ __forceinline__ unsigned img_off(int row, int kk)
{
    return (unsigned)((row >> 3) * 1024 + (kk >> 3) * 128 + (row & 7) * 16 + (kk & 7) * 2);
}

/* bf16 bits of an integer t in [-128, 128] (exact): 1.f x 2^p with p = floor(log2 |t|) */
__device__ __forceinline__ unsigned short bf16_of_int(int t)
{
    const unsigned a = (unsigned)abs(t);
    if (a == 0) return 0;
    const int p = 31 - __clz(a);
    const unsigned bits = ((unsigned)(127 + p) << 7) | ((a << (7 - p)) & 0x7Fu);
    return (unsigned short)(bits | (t < 0 ? 0x8000u : 0u));
}

/* 2^n as a double for n in the normal range */
__device__ __forceinline__ double pow2(int n) { return __longlong_as_double((long long)(1023 + n) << 52); }

/* The slices of one value v of a row (or column) whose largest magnitude is
 * below 2^e: F = rint(v 2^(55-e)) (|F| < 2^55; the cut keeps 55 bits below
 * the row's leading bit), written in balanced base-256 digits F = sum_i t_i
 * 256^(S-1-i), t_i in [-128, 128], i.e. v ~ 2^e sum_i t_i 2^(-7-8i).  dig[i]:
 * the bf16 bits of t_i, i = 0 the leading slice. */
__device__ __forceinline__ void cut_value(double v, int e, unsigned short dig[S])
{
    /* a row of huge or tiny magnitude (outside 2^+-960) scales through ldexp */
    long long F = (e > -960 && e < 960) ? __double2ll_rn(v * pow2(55 - e)) : __double2ll_rn(ldexp(v, 55 - e));
#pragma unroll
    for (int i = S - 1; i > 0; i--) {
        const int t = (int)((F + 128) & 255) - 128;
        dig[i] = bf16_of_int(t);
        F = (F - t) >> 8;
    }
    dig[0] = bf16_of_int((int)F);
}

/* the exponent e with |x| < 2^e for the largest magnitude mx of a row (0 for
 * a zero row) */
__device__ __forceinline__ int row_exponent(double mx)
{
    int e = 0;
    if (mx > 0.0) frexp(mx, &e);
    return e;
}

/* Rows of [Ar | Ai] (m x k, k <= 32 for this pass) cut into S slice images
 * (tile tr = r / 128: image (i * ntr + tr)); ea[r] = the row's exponent.  One
 * warp per row, lane t holds column t; padded rows write zeros. */
__global__ void k_cut_rows(int m, int k, const double2 *__restrict__ A, int lda, unsigned char *__restrict__ img,
                           int *__restrict__ ea, int ntr)
{
    const int r = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5), t = threadIdx.x & 31;
    if (r >= ntr * BM) return;
    double re = 0.0, im = 0.0;
    if (r < m && t < k) {
        const double2 a = A[r + (long long)lda * t];
        re = a.x;
        im = a.y;
    }
    double mx = fmax(fabs(re), fabs(im));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const int e = row_exponent(mx);
    if (t == 0 && r < m) ea[r] = e;
    unsigned short dr[S], di[S];
    cut_value(re, e, dr);
    cut_value(im, e, di);
    const int tr = r / BM, rr = r % BM;
#pragma unroll
    for (int i = 0; i < S; i++) {
        unsigned char *base = img + (size_t)(i * ntr + tr) * AIMG;
        *reinterpret_cast<unsigned short *>(base + img_off(rr, t)) = dr[i];
        *reinterpret_cast<unsigned short *>(base + img_off(rr, KC + t)) = di[i];
    }
}

/* Columns of B (k x n, k <= 32) cut into S slice images of the real
 * [[Br, Bi], [-Bi, Br]]: image (l * ntc + tc) holds, for the complex columns
 * j = 32 tc + jj, row jj = [Br | -Bi] (the Pr column) and row 32 + jj =
 * [Bi | Br] (the Pi column) of the N x K operand; eb[j] = the column's
 * exponent.  One warp per complex column, lane t holds row t. */
__global__ void k_cut_cols(int k, int n, const double2 *__restrict__ B, int ldb, unsigned char *__restrict__ img,
                           int *__restrict__ eb, int ntc)
{
    const int j = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5), t = threadIdx.x & 31;
    if (j >= ntc * BNC) return;
    double re = 0.0, im = 0.0;
    if (j < n && t < k) {
        const double2 b = B[t + (long long)ldb * j];
        re = b.x;
        im = b.y;
    }
    double mx = fmax(fabs(re), fabs(im));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const int e = row_exponent(mx);
    if (t == 0 && j < n) eb[j] = e;
    unsigned short dr[S], di[S];
    cut_value(re, e, dr);
    cut_value(im, e, di);
    const int tc = j / BNC, jj = j % BNC;
#pragma unroll
    for (int l = 0; l < S; l++) {
        unsigned char *base = img + (size_t)(l * ntc + tc) * BIMG;
        *reinterpret_cast<unsigned short *>(base + img_off(jj, t)) = dr[l];
        *reinterpret_cast<unsigned short *>(base + img_off(jj, KC + t)) = (unsigned short)(di[l] ? di[l] ^ 0x8000u : 0u);
        *reinterpret_cast<unsigned short *>(base + img_off(BNC + jj, t)) = di[l];
        *reinterpret_cast<unsigned short *>(base + img_off(BNC + jj, KC + t)) = dr[l];
    }
}

/* X 2^E through FP64 arithmetic, for results outside the normal range (out
 * of line: the compiler would otherwise evaluate it, on GB300's narrow FP64
 * pipe, for every element) */
__device__ __noinline__ double fixed_to_double_slow(long long xt, unsigned xb, int E)
{
    return ldexp(fma((double)xt, 4294967296.0, (double)xb), E);
}

/* The double nearest (ties to even) to X 2^E, X = xt 2^32 + xb (xt signed,
 * |xt| < 2^42; xb in [0, 2^32)), assembled with integer operations; a result
 * outside the normal range goes through FP64 arithmetic instead. */
__device__ __forceinline__ double fixed_to_double(long long xt, unsigned xb, int E)
{
    const bool neg = xt < 0;
    unsigned long long hi, lo;
    if (!neg) {
        hi = (unsigned long long)xt;
        lo = xb;
    } else if (xb) {
        hi = (unsigned long long)(~xt);
        lo = 0x100000000ull - xb;
    } else {
        hi = (unsigned long long)(-xt);
        lo = 0;
    }
    if ((hi | lo) == 0) return 0.0;
    unsigned long long mm;
    bool sticky = false;
    int E2 = E;
    if (hi >> 31) { /* more than 63 bits: the top 64, the rest sticky */
        const int bh = 64 - __clzll((long long)hi), r = bh - 32;
        mm = (hi << (64 - bh)) | (lo >> r);
        sticky = (lo & ((1ull << r) - 1)) != 0;
        E2 += r;
    } else {
        mm = (hi << 32) | lo;
    }
    const int lz = __clzll((long long)mm);
    mm <<= lz;
    E2 -= lz;
    unsigned long long mant = mm >> 11;
    const unsigned rem = (unsigned)(mm & 0x7FFu);
    if ((rem & 0x400u) && ((rem & 0x3FFu) || sticky || (mant & 1ull))) mant++;
    const int bexp = E2 + 11 + 52 + 1023;
    if (bexp < 1 || bexp > 2046) return fixed_to_double_slow(xt, xb, E);
    return __longlong_as_double(
        (long long)(((unsigned long long)neg << 63) + ((unsigned long long)(bexp - 1) << 52) + mant));
}

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, unsigned limit)
{
    for (unsigned it = 0; it < limit; it++) {
        unsigned ok;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}

/* shared-memory operand descriptor: K-major, no swizzle, LBO 128 B (next
 * core matrix along the inner dimension), SBO 1024 B (next 8-row group),
 * descriptor version 1 */
__device__ __forceinline__ uint64_t op_desc(unsigned saddr)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)(128u >> 4) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

/* instruction descriptor, kind::f16: f32 accumulator, bf16 A and B, both
 * K-major, N = 64, M = 128 */
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(unsigned tmem, uint64_t a, uint64_t b, unsigned accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 :
                 : "r"(tmem), "l"(a), "l"(b), "r"(IDESC), "r"(accumulate)
                 : "memory");
}

/* 8 consecutive TMEM columns of this thread's lane */
__device__ __forceinline__ void tmem_ld8(unsigned taddr, float v[8])
{
    unsigned r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 8; j++) v[j] = __uint_as_float(r[j]);
}

constexpr int MMA_THREADS = 256; /* 8 warps: two per TMEM lane quarter in the epilogue */

/* One tile: rows 128 tr.., complex columns 16 tc.. of C; two CTAs per SM, so
 * that one's epilogue runs beside the other's products.  Thread 0 loads every
 * B slice (one mbarrier) and streams the A slices through a ring of three
 * buffers (full / empty mbarriers per buffer; a buffer is refilled once the
 * products that read it have completed, tcgen05.commit); slice i is multiplied
 * with B_l, l = 0 .. S-1-i, into accumulator i + l.  Then the 8 warps read
 * the accumulators back, warp w the TMEM lanes of quarter w % 4 and the
 * complex columns 8 (w / 4) .. + 7.  Every wait is bounded: on a timeout the
 * CTA records error 1, lets its copies in flight land (bounded) and returns
 * through the same epilogue. */
__global__ void __launch_bounds__(MMA_THREADS, 2)
    k_oz_mma(int m, int n, double2 alpha, const unsigned char *__restrict__ aimg, const unsigned char *__restrict__ bimg,
             const int *__restrict__ ea, const int *__restrict__ eb, int ntr, int ntc, double2 *C, int ldc, int *err,
             unsigned wait_limit, int skip_slice)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char *ring = sm, *sB = sm + RING * AIMG;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sB + S * BIMG);
    uint64_t *a_full = bar, *a_empty = bar + RING, *b_full = bar + 2 * RING, *acc_full = bar + 2 * RING + 1;
    unsigned *tslot = reinterpret_cast<unsigned *>(bar + 2 * RING + 2);
    const int tr = blockIdx.x, tc = blockIdx.y;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int b = 0; b < 2 * RING + 2; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar + b)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *tslot;

    if (threadIdx.x == 0) {
        int last[RING]; /* the slice last loaded into each buffer (-1: none) */
#pragma unroll
        for (int r = 0; r < RING; r++) last[r] = -1;
        auto load_a = [&](int i) {
            const int slot = i % RING;
            const unsigned b = smem_u32(a_full + slot);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(AIMG) : "memory");
            last[slot] = i;
            if (i == skip_slice) return; /* the timeout test: a slice that never arrives */
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                             smem_u32(ring + slot * AIMG)),
                         "l"(aimg + (size_t)(i * ntr + tr) * AIMG), "r"(AIMG), "r"(b)
                         : "memory");
        };
        {
            const unsigned b = smem_u32(b_full);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(S * BIMG) : "memory");
            for (int l = 0; l < S; l++)
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        smem_u32(sB + l * BIMG)),
                    "l"(bimg + (size_t)(l * ntc + tc) * BIMG), "r"(BIMG), "r"(b)
                    : "memory");
        }
        for (int i = 0; i < RING && i < S; i++) load_a(i);
        bool ok = mbar_wait(smem_u32(b_full), 0, wait_limit);
        for (int i = 0; i < S && ok; i++) {
            const int slot = i % RING;
            if (!mbar_wait(smem_u32(a_full + slot), (unsigned)((i / RING) & 1), wait_limit)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int l = 0; l + i < S; l++) {
                const unsigned acc = tmem + (unsigned)((i + l) * BN);
#pragma unroll
                for (int ks = 0; ks < KI / 16; ks++)
                    mma_bf16(acc, op_desc(smem_u32(ring + slot * AIMG + ks * 256)),
                             op_desc(smem_u32(sB + l * BIMG + ks * 256)), (i > 0 || ks > 0) ? 1u : 0u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(a_empty + slot))
                         : "memory");
            /* the buffer of slice i - 1 takes slice i - 1 + RING once its products are done */
            const int nx = i - 1 + RING;
            if (i >= 1 && nx < S) {
                const int ps = (i - 1) % RING;
                if (!mbar_wait(smem_u32(a_empty + ps), (unsigned)(((i - 1) / RING) & 1), wait_limit)) {
                    ok = false;
                    break;
                }
                load_a(nx);
            }
        }
        if (!ok) {
            /* record it, and let the copies still in flight land (bounded) */
            atomicExch(err, 1);
            mbar_wait(smem_u32(b_full), 0, wait_limit);
            for (int r = 0; r < RING; r++)
                if (last[r] >= 0) mbar_wait(smem_u32(a_full + r), (unsigned)((last[r] / RING) & 1), wait_limit);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(acc_full))
                     : "memory");
    }
    __syncwarp();
    const bool done = mbar_wait(smem_u32(acc_full), 0, wait_limit);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!done) {
        if (lane == 0) atomicExch(err, 2);
    } else {
        const int q = warp & 3, g = warp >> 2;
        const int row = tr * BM + q * 32 + lane;
        const unsigned lane_base = tmem + ((unsigned)(q * 32) << 16);
        const int er = row < m ? ea[row] : 0;
        /* X = sum_d acc_d 256^(S-1-d) exactly: int32 pairs (acc_1, acc_2),
         * (acc_3, acc_4), (acc_5, acc_6) (each below 2^31), then two int64
         * halves th = acc_0 2^16 + p12 (below 2^40) and tl = p34 2^16 + p56
         * (below 2^48): X = th 2^32 + tl; value X 2^(er + ec - 62) */
        static_assert(S == 7, "the pairing below is written for 7 slices");
        int a0[2][8], p12[2][8], p34[2][8], p56[2][8];
#pragma unroll
        for (int h = 0; h < 2; h++) { /* Pr, then Pi */
            const unsigned base = lane_base + (unsigned)(h * BNC + g * 8);
            float v[8], w[8];
            tmem_ld8(base, v);
#pragma unroll
            for (int j = 0; j < 8; j++) a0[h][j] = __float2int_rn(v[j]);
#pragma unroll
            for (int pr = 0; pr < 3; pr++) {
                tmem_ld8(base + (unsigned)((1 + 2 * pr) * BN), v);
                tmem_ld8(base + (unsigned)((2 + 2 * pr) * BN), w);
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int q2 = __float2int_rn(v[j]) * 256 + __float2int_rn(w[j]);
                    if (pr == 0) p12[h][j] = q2;
                    else if (pr == 1) p34[h][j] = q2;
                    else p56[h][j] = q2;
                }
            }
        }
        /* C += alpha * value; a real alpha (the layer transfer's -1 and 1)
         * gets a loop of its own, so that no element evaluates the complex
         * form's extra FP64 multiply-adds */
        auto update = [&](auto real_alpha) {
            if (row >= m) return;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int col = tc * BNC + g * 8 + j;
                if (col < n) {
                    const int E = er + eb[col] - 14 - 8 * (S - 1);
                    double x[2];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const long long th = ((long long)a0[h][j] << 16) + p12[h][j];
                        const long long tl = ((long long)p34[h][j] << 16) + p56[h][j];
                        x[h] = fixed_to_double(th + (tl >> 32), (unsigned)tl, E);
                    }
                    double2 *c = C + row + (long long)ldc * col;
                    double2 v = *c;
                    if (decltype(real_alpha)::value) {
                        v.x = fma(alpha.x, x[0], v.x);
                        v.y = fma(alpha.x, x[1], v.y);
                    } else {
                        v.x = fma(alpha.x, x[0], fma(-alpha.y, x[1], v.x));
                        v.y = fma(alpha.x, x[1], fma(alpha.y, x[0], v.y));
                    }
                    *c = v;
                }
            }
        };
        if (alpha.y == 0.0) update(std::true_type{});
        else update(std::false_type{});
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

} // namespace

size_t tc_workspace_bytes(int m, int n)
{
    const size_t ntr = (size_t)((m + BM - 1) / BM), ntc = (size_t)((n + BNC - 1) / BNC);
    const size_t img = (size_t)S * (ntr * AIMG + ntc * BIMG);
    return img + sizeof(int) * (ntr * BM + ntc * BNC) + 256;
}

bool tc_available()
{
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return optin >= SMEM;
}

int zgemm_acc_tc(int m, int n, int k, double2 alpha, const double2 *A, int lda, const double2 *B, int ldb, double2 *C,
                 int ldc, const GemmCtx &g, cudaStream_t st)
{
    if (m <= 0 || n <= 0 || k <= 0) return SMAT_OK;
    const int ntr = (m + BM - 1) / BM, ntc = (n + BNC - 1) / BNC;
    if (!g.ws || g.ws_bytes < tc_workspace_bytes(m, n) || !g.err)
        return smat_fail(SMAT_EINVAL, "zgemm (tensor cores): workspace of %zu bytes for %d x %d, %zu given",
                         tc_workspace_bytes(m, n), m, n, g.ws_bytes);
    if (cudaFuncSetAttribute(k_oz_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM) != cudaSuccess)
        return smat_fail(SMAT_ECUDA, "zgemm (tensor cores): %d bytes of shared memory refused", SMEM);
    unsigned char *aimg = static_cast<unsigned char *>(g.ws);
    unsigned char *bimg = aimg + (size_t)S * ntr * AIMG;
    int *ea = reinterpret_cast<int *>(bimg + (size_t)S * ntc * BIMG);
    int *eb = ea + ntr * BM;
    for (int k0 = 0; k0 < k; k0 += KC) {
        const int kp = k - k0 < KC ? k - k0 : KC;
        k_cut_rows<<<(ntr * BM + 7) / 8, 256, 0, st>>>(m, kp, A + (long long)lda * k0, lda, aimg, ea, ntr);
        k_cut_cols<<<(ntc * BNC + 7) / 8, 256, 0, st>>>(kp, n, B + k0, ldb, bimg, eb, ntc);
        k_oz_mma<<<dim3((unsigned)ntr, (unsigned)ntc), MMA_THREADS, SMEM, st>>>(
            m, n, alpha, aimg, bimg, ea, eb, ntr, ntc, C, ldc, g.err, g.wait_limit ? g.wait_limit : WAIT_LIMIT,
            g.skip_pair);
        if (cudaPeekAtLastError() != cudaSuccess)
            return smat_fail(SMAT_ECUDA, "zgemm (tensor cores) launch: %s", cudaGetErrorString(cudaGetLastError()));
    }
    return SMAT_OK;
}

} // namespace dense
} // namespace smat
