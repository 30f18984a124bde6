/*
 * Mode-overlap projection on the GPU: the S-parameter extraction of the
 * reference S_calc (FDTDsplitfieldMetal.c:437-445),
 *
 *   S[v][c] = sum_r conj(tilXi[r, c]) * x_v[r],
 *   x_v = (HB_x, HB_y, -EB_y, EB_x) of DFT plane v (4*npix rows),
 *
 * for ncols columns of tilde-Xi and nvec DFT planes (e.g. all wavelengths of
 * one monitor plane) at once, in FP64.  Two passes: each block sums a fixed
 * range of rows into a partial (scratch memory of nblk * nvec * ncols complex
 * values), then one thread per (v, c) adds the partials in block order.  The
 * grid is a function of npix only, so a result is the same bits on every call.
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "trace.cuh"
#include "fdtd_internal.cuh"
#include "plan_internal.cuh"
#include "host_internal.h"
#include "smatran_fdtd.h"

namespace smat {

constexpr int OV_THREADS = 256;

int overlap_blocks(int npix)
{
    const long long rows = 4LL * npix;
    long long nb = (rows + 4 * OV_THREADS - 1) / (4 * OV_THREADS);
    return (int)(nb < 1 ? 1 : (nb > 64 ? 64 : nb));
}

/* dft: plane v at dft + v*vec_stride (complex), components (Hx, Hy, Ex, Ey) x npix */
__global__ void k_overlap_partial(int npix, int ncols, long long vec_stride, const double2 *__restrict__ t,
                                  const double2 *__restrict__ dft, double2 *__restrict__ part)
{
    __shared__ double2 red[OV_THREADS];
    const int nblk = gridDim.x, blk = blockIdx.x, c = blockIdx.y, v = blockIdx.z;
    const long long rows = 4LL * npix;
    const long long chunk = (rows + nblk - 1) / nblk;
    const long long r0 = blk * chunk, r1 = min(rows, r0 + chunk);
    const double2 *tc = t + (long long)c * rows;
    const double2 *x = dft + (long long)v * vec_stride;
    double sr = 0.0, si = 0.0;
    for (long long r = r0 + threadIdx.x; r < r1; r += OV_THREADS) {
        const int comp = (int)(r / npix);
        const long long px = r - (long long)comp * npix;
        /* row blocks of tilde-Xi: HB_x, HB_y, -EB_y, EB_x */
        double2 xv;
        if (comp == 0) xv = x[px];
        else if (comp == 1) xv = x[npix + px];
        else if (comp == 2) {
            xv = x[3LL * npix + px];
            xv.x = -xv.x;
            xv.y = -xv.y;
        } else xv = x[2LL * npix + px];
        const double2 a = tc[r];
        /* conj(a) * xv */
        sr += a.x * xv.x + a.y * xv.y;
        si += a.x * xv.y - a.y * xv.x;
    }
    red[threadIdx.x] = make_double2(sr, si);
    __syncthreads();
    for (int s = OV_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            red[threadIdx.x].x += red[threadIdx.x + s].x;
            red[threadIdx.x].y += red[threadIdx.x + s].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[((long long)v * ncols + c) * nblk + blk] = red[0];
}

__global__ void k_overlap_final(int ncols, int nvec, int nblk, const double2 *__restrict__ part,
                                double2 *__restrict__ S)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncols * nvec) return;
    double sr = 0.0, si = 0.0;
    for (int b = 0; b < nblk; b++) {
        const double2 q = part[(long long)i * nblk + b];
        sr += q.x;
        si += q.y;
    }
    S[i] = make_double2(sr, si);
}

int overlap_launch(int npix, int ncols, int nvec, long long vec_stride, const double *tilXi, const double *dft,
                   double *S, double2 *scratch, cudaStream_t st)
{
    const int nblk = overlap_blocks(npix);
    dim3 g1(nblk, ncols, nvec);
    k_overlap_partial<<<g1, OV_THREADS, 0, st>>>(npix, ncols, vec_stride, (const double2 *)tilXi,
                                                 (const double2 *)dft, scratch);
    const int n = ncols * nvec;
    k_overlap_final<<<(n + 127) / 128, 128, 0, st>>>(ncols, nvec, nblk, scratch, (double2 *)S);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return smat_fail(SMAT_ECUDA, "overlap launch: %s", cudaGetErrorString(e));
    return SMAT_OK;
}

} // namespace smat

using namespace smat;

static int overlap_args_ok(int npix, int ncols, int nvec, long long vec_stride, const double *t, const double *d,
                           const double *S)
{
    if (npix <= 0 || ncols <= 0 || nvec <= 0 || !t || !d || !S || ncols > 65535 || nvec > 65535)
        return smat_fail(SMAT_EINVAL, "overlap: bad arguments");
    if (nvec > 1 && vec_stride < 4LL * npix) return smat_fail(SMAT_EINVAL, "overlap: vec_stride < 4*npix");
    return SMAT_OK;
}

extern "C" int smat_overlap(int npix, int ncols, int nvec, long long vec_stride, const double *tilXi,
                            const double *dft, double *S, void *stream)
{
    smat_clear_error();
    int rc = overlap_args_ok(npix, ncols, nvec, vec_stride, tilXi, dft, S);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)overlap_blocks(npix) * ncols * nvec;
    double2 *scratch = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&scratch, n * sizeof(double2), st);
    if (e != cudaSuccess) return smat_fail(SMAT_ENOMEM, "overlap scratch: %s", cudaGetErrorString(e));
    rc = overlap_launch(npix, ncols, nvec, vec_stride, tilXi, dft, S, scratch, st);
    cudaFreeAsync(scratch, st);
    return rc;
}

/* DFT accumulator pointer of a plan (used by the plan-level helper below) */
extern "C" int smat_fdtd_dft_device(smat_fdtd_plan *plan, int b, int f, int q, const double **ptr, long long *fstride);

extern "C" int smat_fdtd_overlap(smat_fdtd_plan *plan, int b, int q, int ncols, const double *tilXi_host,
                                 double *S_host)
{
    smat::TraceRange trace_("smat_fdtd_overlap");
    smat_clear_error();
    const double *acc = nullptr;
    long long fstride = 0;
    int L[4], nb = 0;
    int rc = smat_fdtd_info(plan, L, nullptr, nullptr, &nb);
    if (rc) return rc;
    rc = smat_fdtd_dft_device(plan, b, 0, q, &acc, &fstride);
    if (rc) return rc;
    const int npix = L[0] * L[1];
    int nfreq = 0;
    rc = smat_fdtd_dft_count(plan, &nfreq, nullptr);
    if (rc) return rc;
    if (ncols <= 0 || !tilXi_host || !S_host) return smat_fail(SMAT_EINVAL, "fdtd_overlap: bad arguments");
    double *dt = nullptr, *dS = nullptr;
    const size_t tn = (size_t)ncols * 4 * npix * 2, sn = (size_t)nfreq * ncols * 2;
    if (cudaMalloc((void **)&dt, tn * 8) != cudaSuccess || cudaMalloc((void **)&dS, sn * 8) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(dt);
        return smat_fail(SMAT_ENOMEM, "fdtd_overlap: device buffers");
    }
    rc = SMAT_OK;
    plan->h2d_bytes += (long long)tn * 8;
    if (cudaMemcpy(dt, tilXi_host, tn * 8, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = smat_fail(SMAT_ECUDA, "fdtd_overlap: upload");
    if (!rc) rc = smat_fdtd_sync(plan);
    if (!rc) rc = smat_overlap(npix, ncols, nfreq, fstride, dt, acc, dS, nullptr);
    if (!rc) plan->d2h_bytes += (long long)sn * 8;
    if (!rc && cudaMemcpy(S_host, dS, sn * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = smat_fail(SMAT_ECUDA, "fdtd_overlap: download");
    cudaFree(dt);
    cudaFree(dS);
    return rc;
}

/* ---------------------------------------------------------------------------
 * Allocation-free variant of smat_overlap.
 *
 * Some callers cannot allocate device memory while they extract S parameters:
 * a host process whose memory pool is reserved by a framework that owns the
 * device (and forbids others to call cudaMalloc/cudaMallocAsync), or a
 * real-time loop that must not risk an allocation failure after start-up.
 * smat_overlap_noalloc does the same projection with its block partial sums in
 * a fixed device array that lives in this library's module, so it never
 * allocates.  The array holds SMAT_OVERLAP_NOALLOC_MAX complex partial sums
 * (1 MiB) on every device that loads the library, until the process exits.
 * ------------------------------------------------------------------------- */
static __device__ __align__(256) double2 g_overlap_scratch[SMAT_OVERLAP_NOALLOC_MAX];

namespace {
constexpr int MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
/* the array's device address per device, and the context it was taken in: a
 * context destroyed and re-created (cudaDeviceReset, a primary context
 * released by its last user) reloads the module, so the address is looked up
 * again when the current context is not the one it was taken in */
double2 *g_noalloc_addr[MAX_DEVICES];
CUcontext g_noalloc_ctx[MAX_DEVICES];

typedef CUresult (*ctx_get_current_fn)(CUcontext *);
ctx_get_current_fn ctx_get_current()
{
    static ctx_get_current_fn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &ptr, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (ctx_get_current_fn)ptr;
        else
            cudaGetLastError();
    }
    return fn;
}
} // namespace

extern "C" int smat_overlap_noalloc(int npix, int ncols, int nvec, long long vec_stride, const double *tilXi,
                                    const double *dft, double *S, void *stream)
{
    smat_clear_error();
    int rc = overlap_args_ok(npix, ncols, nvec, vec_stride, tilXi, dft, S);
    if (rc) return rc;
    const long long need = (long long)overlap_blocks(npix) * ncols * nvec;
    if (need > SMAT_OVERLAP_NOALLOC_MAX)
        return smat_fail(SMAT_EINVAL,
                         "overlap_noalloc: %lld partial sums needed (ncols*nvec*%d blocks), the static scratch "
                         "holds %d; use smat_overlap or fewer columns/planes per call",
                         need, overlap_blocks(npix), SMAT_OVERLAP_NOALLOC_MAX);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return smat_fail(SMAT_ECUDA, "overlap_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES) return smat_fail(SMAT_EINVAL, "overlap_noalloc: device %d out of range", dev);
    double2 *scratch = nullptr;
    {
        /* once per device (and context), with that device current: the device
         * address of the static array (the host-side symbol is not a device
         * address) */
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        CUcontext ctx = nullptr;
        ctx_get_current_fn get = ctx_get_current();
        const bool known_ctx = get && get(&ctx) == CUDA_SUCCESS && ctx;
        if (!g_noalloc_addr[dev] || !known_ctx || ctx != g_noalloc_ctx[dev]) {
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_overlap_scratch);
            if (e != cudaSuccess || !ptr)
                return smat_fail(SMAT_ECUDA, "overlap_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            g_noalloc_addr[dev] = (double2 *)ptr;
            g_noalloc_ctx[dev] = known_ctx ? ctx : nullptr;
        }
        scratch = g_noalloc_addr[dev];
    }
    /* every partial the second pass reads is written by the first pass of the
     * same call, so the array needs no clearing between calls */
    return overlap_launch(npix, ncols, nvec, vec_stride, tilXi, dft, S, scratch, (cudaStream_t)stream);
}
