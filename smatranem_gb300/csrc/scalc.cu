/*
 * Frequency-domain S matrix by layer transfer on the GPU: the reference's
 * Smat/Scalc.c (main :74-96) with its dense steps on the device.
 *
 * State per direction (iway = +1 bottom -> top, -1 top -> bottom), NA =
 * 2*L0*L1, No = modes of the starting port: F01 ((No+NA) x No), B01
 * ((No+NA) x NA), F2 (NA x No), B2 (NA x NA), all complex FP64 in HBM.
 *   set_iniMat (:407-458): the starting port's full mode matrix Phi;
 *   per half layer (initial_calc :192-221, scattering_calc :227-261,
 *   final_calc :269-306): F2 <- field rows of F01, B2 <- field rows of B01
 *   + i*iway*(maa or mbb of the layer), field rows of B01 <- 1, inv_process;
 *   set_finMat (:461-517): project on the ending port's dual modes;
 *   inv_process (:316-400): B01 <- B01 B2^{-1} (LU with partial pivoting of
 *   B2^T, the zgesv of the reference), F01 <- F01 - B01 F2, F2 = 0, B2 = 1.
 * maa / mbb are never formed: k_add_op adds each row's stencil coefficients
 * (those of set_M :716-790) straight into B2.
 */
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "dense_z.cuh"
#include "host_internal.h"
#include "smatran_fdtd.h"
#include "trace.cuh"

namespace {

using smat::dense::getrf;
using smat::dense::getrs;
using smat::dense::transpose;
using smat::dense::zgemm_acc;

struct Geo {
    int L0, L1, NA1;
    double s0, s1, e0, e1;  // set_D's diagonal and wrap coefficients (as in the mode solver)
};

__device__ __forceinline__ double cw(int i, int La, double e) { return i < La - 1 ? 1.0 : e; }

/* B2[r, col] += i*sgn * M[r, col] over the stencil of row r; which = 0: maa,
 * 1: mbb; V = 6*NA1 complex set_V values.  One thread per row. */
__global__ void k_add_op(double2 *B2, int ld, Geo g, const double2 *__restrict__ V, int which, double sgn)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int NA1 = g.NA1;
    if (r >= 2 * NA1) return;
    const int comp = r / NA1, p = r % NA1;
    const int i0 = p % g.L0, i1 = p / g.L0;
    double2 *row = B2 + r;
    auto pt = [&](int j0, int j1) {
        j0 = ((j0 % g.L0) + g.L0) % g.L0;
        j1 = ((j1 % g.L1) + g.L1) % g.L1;
        return j0 + g.L0 * j1;
    };
    auto emit = [&](int c, int q, double2 v) {  // += i*sgn*v
        double2 *e = row + (long long)ld * (c * NA1 + q);
        e->x -= sgn * v.y;
        e->y += sgn * v.x;
    };
    auto sc = [](double2 v, double f) { return make_double2(v.x * f, v.y * f); };
    auto c0 = [&](int j0) { return cw(((j0 % g.L0) + g.L0) % g.L0, g.L0, g.e0); };
    auto c1 = [&](int j1) { return cw(((j1 % g.L1) + g.L1) % g.L1, g.L1, g.e1); };
    if (which == 0) {
        /* curl terms w(q) = V2(q) (s1 x0(q) + c1 x0(q+e1) - s0 x1(q) - c0 x1(q+e0)), times f */
        auto wt = [&](int j0, int j1, double2 f) {
            const int q = pt(j0, j1);
            emit(0, q, sc(f, g.s1));
            emit(0, pt(j0, j1 + 1), sc(f, c1(j1)));
            emit(1, q, sc(f, -g.s0));
            emit(1, pt(j0 + 1, j1), sc(f, -c0(j0)));
        };
        const double2 *V2 = V + 2 * NA1;
        if (comp == 0) {  // V0 x0 + Ddown1 w
            emit(0, p, V[p]);
            wt(i0, i1, sc(V2[p], -g.s1));
            const int q = pt(i0, i1 - 1);
            wt(i0, i1 - 1, sc(V2[q], -c1(i1 - 1)));
        } else {  // V1 x1 - Ddown0 w
            emit(1, p, V[NA1 + p]);
            wt(i0, i1, sc(V2[p], g.s0));
            const int q = pt(i0 - 1, i1);
            wt(i0 - 1, i1, sc(V2[q], c0(i0 - 1)));
        }
    } else {
        /* u(q) = V5(q) (-s0 y0(q) - c0(q-e0) y0(q-e0) - s1 y1(q) - c1(q-e1) y1(q-e1)), times f */
        auto ut = [&](int j0, int j1, double2 f) {
            emit(0, pt(j0, j1), sc(f, -g.s0));
            emit(0, pt(j0 - 1, j1), sc(f, -c0(j0 - 1)));
            emit(1, pt(j0, j1), sc(f, -g.s1));
            emit(1, pt(j0, j1 - 1), sc(f, -c1(j1 - 1)));
        };
        const double2 *V5 = V + 5 * NA1;
        if (comp == 0) {  // V3 y0 + Dup0 u
            emit(0, p, V[3 * NA1 + p]);
            ut(i0, i1, sc(V5[p], g.s0));
            ut(i0 + 1, i1, sc(V5[pt(i0 + 1, i1)], c0(i0)));
        } else {  // V4 y1 + Dup1 u
            emit(1, p, V[4 * NA1 + p]);
            ut(i0, i1, sc(V5[p], g.s1));
            ut(i0, i1 + 1, sc(V5[pt(i0, i1 + 1)], c1(i1)));
        }
    }
}

/* dst (m x n, ldd) = src (ldsrc) */
__global__ void k_copy2d(int m, int n, const double2 *__restrict__ src, int lds, double2 *__restrict__ dst, int ldd)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m * n) return;
    const int r = (int)(t % m), c = (int)(t / m);
    dst[r + (long long)ldd * c] = src[r + (long long)lds * c];
}

/* dst (m x n) = diag * identity (diag 0: zero) */
__global__ void k_set2d(int m, int n, double2 *dst, int ldd, double diag)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m * n) return;
    const int r = (int)(t % m), c = (int)(t / m);
    dst[r + (long long)ldd * c] = make_double2(r == c ? diag : 0.0, 0.0);
}

/* the full mode matrix of set_Phi (:521-551) / set_tilPhi (:555-595) from Xi
 * (2NA x 2NA, Mcalc's column order); kind 0: Phi, 1: tilPhi */
__global__ void k_phi(const double2 *__restrict__ Xi, double2 *__restrict__ P, int NA, int iway, int nimag, int kind)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int N2 = 2 * NA;
    if (t >= (long long)N2 * N2) return;
    const int r = (int)(t % N2), col = (int)(t / N2);
    const int j = col % NA, hi = col >= NA;
    const int rr = (r + NA) % N2;  // the file row that lands on row r after the half rotation
    auto X = [&](int row, int c) { return Xi[row + (long long)N2 * c]; };
    auto neg = [](double2 v) { return make_double2(-v.x, -v.y); };
    double2 v;
    if (kind == 0) {
        v = iway == 1 ? X(r, col) : X(rr, hi ? j : j + NA);
    } else if (iway == 1) {
        if (j < nimag) v = hi ? neg(X(rr, j + NA)) : X(rr, j);
        else v = hi ? X(rr, j) : X(rr, j + NA);
    } else {
        if (j < nimag) v = hi ? X(r, j) : neg(X(r, j + NA));
        else v = hi ? X(r, j + NA) : X(r, j);
    }
    P[r + (long long)N2 * col] = v;
}

#define SCK(call)                                                                                                      \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) return smat_fail(SMAT_ECUDA, "%s: %s", #call, cudaGetErrorString(e_));                \
    } while (0)
#define RC(call)                                                                                                       \
    do {                                                                                                               \
        int r_ = (call);                                                                                               \
        if (r_) return r_;                                                                                             \
    } while (0)

struct Transfer {
    Geo g{};
    int NA = 0, No = 0, ldF = 0;
    cudaStream_t st = nullptr;
    double2 *F01 = nullptr, *B01 = nullptr, *F2 = nullptr, *B2 = nullptr, *W1 = nullptr, *W2 = nullptr;
    double2 *Xi = nullptr, *P = nullptr, *PH = nullptr, *FB = nullptr, *Cm = nullptr, *V = nullptr;
    int *ipiv = nullptr, *dinfo = nullptr;
    int solves = 0;
    smat::dense::GemmCtx gm{0, nullptr, 0, nullptr}; /* how the multiply-adds run */

    ~Transfer()
    {
        if (st) cudaStreamSynchronize(st);
        smat::dense::gemm_ctx_release(gm);
        for (double2 *b : {F01, B01, F2, B2, W1, W2, Xi, P, PH, FB, Cm, V}) cudaFree(b);
        cudaFree(ipiv);
        cudaFree(dinfo);
        if (st) cudaStreamDestroy(st);
    }
    static unsigned blocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }
    int copy2d(int m, int n, const double2 *s, int lds, double2 *d, int ldd)
    {
        if ((long long)m * n == 0) return SMAT_OK;
        k_copy2d<<<blocks((long long)m * n, 256), 256, 0, st>>>(m, n, s, lds, d, ldd);
        return cudaPeekAtLastError() == cudaSuccess ? SMAT_OK : smat_fail(SMAT_ECUDA, "k_copy2d launch");
    }
    int set2d(int m, int n, double2 *d, int ldd, double diag)
    {
        if ((long long)m * n == 0) return SMAT_OK;
        k_set2d<<<blocks((long long)m * n, 256), 256, 0, st>>>(m, n, d, ldd, diag);
        return cudaPeekAtLastError() == cudaSuccess ? SMAT_OK : smat_fail(SMAT_ECUDA, "k_set2d launch");
    }
    /* inv_process :316-400 */
    int inv_process()
    {
        RC(transpose(NA, NA, B2, NA, W1, NA, false, st));
        RC(transpose(No + NA, NA, B01, ldF, W2, NA, false, st));
        RC(getrf(NA, W1, NA, ipiv, dinfo, &gm, st));
        RC(getrs(NA, No + NA, W1, NA, ipiv, W2, NA, &gm, st));
        RC(transpose(NA, No + NA, W2, NA, B01, ldF, false, st));
        RC(zgemm_acc(No + NA, No, NA, make_double2(-1.0, 0.0), B01, ldF, F2, NA, F01, ldF, &gm, st));
        RC(set2d(NA, No, F2, NA, 0.0));
        RC(set2d(NA, NA, B2, NA, 1.0));
        solves++;
        return SMAT_OK;
    }
    /* F2 <- field rows of F01, which become 0 */
    int shift()
    {
        RC(copy2d(NA, No, F01 + No, ldF, F2, NA));
        return set2d(NA, No, F01 + No, ldF, 0.0);
    }
    /* B2 <- field rows of B01 + i*iway*M; field rows of B01 <- 1; eliminate */
    int step(int which, int iway)
    {
        RC(copy2d(NA, NA, B01 + No, ldF, B2, NA));
        k_add_op<<<blocks(NA, 128), 128, 0, st>>>(B2, NA, g, V, which, (double)iway);
        SCK(cudaPeekAtLastError());
        RC(set2d(NA, NA, B01 + No, ldF, 1.0));
        return inv_process();
    }
    int upload_layer(const std::vector<std::complex<double>> &v)
    {
        SCK(cudaMemcpyAsync(V, v.data(), v.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
        return SMAT_OK;
    }
};

/* Scalc's set_V (:838-880): omega * value, rows 2 and 5 inverted as conj(z)/|z|^2;
 * returns the count of entries with a nonzero imaginary part */
int scalc_V(const double *med, long long NA1, double omega, std::vector<std::complex<double>> &v)
{
    v.resize(6 * NA1);
    int comp = 0;
    for (long long k = 0; k < 6 * NA1; k++) {
        std::complex<double> z(med[2 * k] * omega, med[2 * k + 1] * omega);
        const int row = (int)(k / NA1);
        if (row == 2 || row == 5) z = std::conj(z) / (z.real() * z.real() + z.imag() * z.imag());
        v[k] = z;
        if (z.imag() != 0.0) comp++;
    }
    return comp;
}

/* one direction (main :74-94); meds: nlayers layers starting at istart in the
 * direction of travel; Xs / Xe: start / end port Xi (host) */
int one_way(Transfer &T, int iway, int nlayers, const double *const *meds, double omega, const double *Xs,
            const double *Xe, int No, int Nimag, std::vector<std::complex<double>> &F01h,
            std::vector<std::complex<double>> &B01h)
{
    const int NA = T.NA, N2 = 2 * NA;
    const long long NA1 = T.g.NA1;
    T.No = No;
    T.ldF = No + NA;
    std::vector<std::complex<double>> v;
    /* set_iniMat :407-458 */
    SCK(cudaMemcpyAsync(T.Xi, Xs, sizeof(double2) * (size_t)N2 * N2, cudaMemcpyHostToDevice, T.st));
    k_phi<<<Transfer::blocks((long long)N2 * N2, 256), 256, 0, T.st>>>(T.Xi, T.P, NA, iway, 0, 0);
    SCK(cudaPeekAtLastError());
    RC(T.set2d(No, No, T.F01, T.ldF, 0.0));
    RC(T.set2d(No, NA, T.B01, T.ldF, 1.0));  /* top rows of B01: identity in the first No columns */
    RC(T.copy2d(NA, No, T.P, N2, T.F01 + No, T.ldF));
    RC(T.copy2d(NA, No, T.P + NA, N2, T.F2, NA));
    RC(T.copy2d(NA, NA, T.P + (long long)N2 * NA, N2, T.B01 + No, T.ldF));
    RC(T.copy2d(NA, NA, T.P + NA + (long long)N2 * NA, N2, T.B2, NA));
    RC(T.inv_process());
    /* initial_calc :192-221 */
    RC(T.shift());
    if (scalc_V(meds[0], NA1, omega, v)) return smat_fail(SMAT_EINVAL, "V is not real in initial_calc");
    RC(T.upload_layer(v));
    RC(T.step(iway > 0 ? 1 : 0, iway));
    /* scattering_calc :227-261 */
    for (int l = 1; l + 1 < nlayers; l++) {
        scalc_V(meds[l], NA1, omega, v);  /* a lossy inner layer is allowed (a warning in the reference) */
        RC(T.upload_layer(v));
        for (int sub = 0; sub < 2; sub++) {
            RC(T.shift());
            const int i_shift = ((1 - iway) / 2 + sub) % 2;
            RC(T.step(i_shift, iway));
        }
    }
    /* final_calc :269-306 */
    RC(T.shift());
    if (scalc_V(meds[nlayers - 1], NA1, omega, v)) return smat_fail(SMAT_EINVAL, "V is not real in final_calc");
    RC(T.upload_layer(v));
    RC(T.step(iway > 0 ? 0 : 1, iway));
    /* set_finMat :461-517: C = tilPhi^H [F01 field rows, B01 field rows; F2, B2] */
    SCK(cudaMemcpyAsync(T.Xi, Xe, sizeof(double2) * (size_t)N2 * N2, cudaMemcpyHostToDevice, T.st));
    k_phi<<<Transfer::blocks((long long)N2 * N2, 256), 256, 0, T.st>>>(T.Xi, T.P, NA, iway, Nimag, 1);
    SCK(cudaPeekAtLastError());
    RC(transpose(N2, N2, T.P, N2, T.PH, N2, true, T.st));
    const int nc = No + NA;
    RC(T.copy2d(NA, No, T.F01 + No, T.ldF, T.FB, N2));
    RC(T.copy2d(NA, No, T.F2, NA, T.FB + NA, N2));
    RC(T.copy2d(NA, NA, T.B01 + No, T.ldF, T.FB + (long long)N2 * No, N2));
    RC(T.copy2d(NA, NA, T.B2, NA, T.FB + NA + (long long)N2 * No, N2));
    RC(T.set2d(N2, nc, T.Cm, N2, 0.0));
    RC(zgemm_acc(N2, nc, N2, make_double2(1.0, 0.0), T.PH, N2, T.FB, N2, T.Cm, N2, &T.gm, T.st));
    RC(T.copy2d(NA, No, T.Cm, N2, T.F01 + No, T.ldF));
    RC(T.copy2d(NA, No, T.Cm + NA, N2, T.F2, NA));
    RC(T.copy2d(NA, NA, T.Cm + (long long)N2 * No, N2, T.B01 + No, T.ldF));
    RC(T.copy2d(NA, NA, T.Cm + NA + (long long)N2 * No, N2, T.B2, NA));
    RC(T.inv_process());
    /* the rows Smat_calc reads: the top No + Nimag rows of F01 and B01 */
    const int N = No + Nimag;
    F01h.assign((size_t)N * No, 0.0);
    B01h.assign((size_t)N * NA, 0.0);
    for (int c = 0; c < No; c++)
        SCK(cudaMemcpyAsync(&F01h[(size_t)N * c], T.F01 + (long long)T.ldF * c, sizeof(double2) * N,
                            cudaMemcpyDeviceToHost, T.st));
    for (int c = 0; c < Nimag && c < NA; c++)
        SCK(cudaMemcpyAsync(&B01h[(size_t)N * c], T.B01 + (long long)T.ldF * c, sizeof(double2) * N,
                            cudaMemcpyDeviceToHost, T.st));
    SCK(cudaStreamSynchronize(T.st));
    return SMAT_OK;
}

} // namespace

extern "C" int smat_scalc(int L0, int L1, const int BoundC[2], double omega, int nlayers, const double *meds,
                          const double *XiB, int nB, const double *XiT, int nT, int both_ways, double *S,
                          smat_scalc_info *info)
{
    smat::TraceRange trace_("smat_scalc");
    const auto t0 = std::chrono::steady_clock::now();
    if (L0 <= 0 || L1 <= 0 || (long long)L0 * L1 > 8192)
        return smat_fail(SMAT_EINVAL, "smat_scalc: lattice %d x %d (dense transfer: 2*L0*L1 <= 16384)", L0, L1);
    if (!BoundC || BoundC[0] < -1 || BoundC[0] > 1 || BoundC[1] < -1 || BoundC[1] > 1)
        return smat_fail(SMAT_EINVAL, "smat_scalc: BoundC");
    if (nlayers < 2 || !meds || !XiB || !XiT || !S) return smat_fail(SMAT_EINVAL, "smat_scalc: nlayers = %d", nlayers);
    const int NA1 = L0 * L1, NA = 2 * NA1, N2 = 2 * NA;
    if (nB < 1 || nT < 1 || nB > NA || nT > NA) return smat_fail(SMAT_EINVAL, "smat_scalc: modes %d, %d", nB, nT);
    if (!(omega > 0) || !std::isfinite(omega)) return smat_fail(SMAT_EINVAL, "smat_scalc: omega = %g", omega);
    const int Nmax = std::max(nB, nT);
    const size_t ldF = (size_t)Nmax + NA;
    /* one transfer state per direction: device matrices, stream, product workspace */
    auto setup = [&](Transfer &T) {
        T.NA = NA;
        T.g.L0 = L0;
        T.g.L1 = L1;
        T.g.NA1 = NA1;
        T.g.s0 = L0 > 1 ? -1.0 : (double)BoundC[0];
        T.g.s1 = L1 > 1 ? -1.0 : (double)BoundC[1];
        T.g.e0 = L0 > 1 ? (double)BoundC[0] : 0.0;
        T.g.e1 = L1 > 1 ? (double)BoundC[1] : 0.0;
        SCK(cudaStreamCreateWithFlags(&T.st, cudaStreamNonBlocking));
        auto alloc = [&](double2 **p, size_t n) {
            if (cudaMalloc((void **)p, n * sizeof(double2)) != cudaSuccess) {
                cudaGetLastError();
                return smat_fail(SMAT_ENOMEM, "smat_scalc: %zu bytes of device memory", n * sizeof(double2));
            }
            return SMAT_OK;
        };
        RC(alloc(&T.F01, ldF * Nmax));
        RC(alloc(&T.B01, ldF * NA));
        RC(alloc(&T.F2, (size_t)NA * Nmax));
        RC(alloc(&T.B2, (size_t)NA * NA));
        RC(alloc(&T.W1, (size_t)NA * NA));
        RC(alloc(&T.W2, (size_t)NA * ldF));
        RC(alloc(&T.Xi, (size_t)N2 * N2));
        RC(alloc(&T.P, (size_t)N2 * N2));
        RC(alloc(&T.PH, (size_t)N2 * N2));
        RC(alloc(&T.FB, (size_t)N2 * ldF));
        RC(alloc(&T.Cm, (size_t)N2 * ldF));
        RC(alloc(&T.V, 6 * (size_t)NA1));
        SCK(cudaMalloc(&T.ipiv, sizeof(int) * NA));
        SCK(cudaMalloc(&T.dinfo, sizeof(int)));
        SCK(cudaMemsetAsync(T.dinfo, 0, sizeof(int), T.st));
        /* products up to 2NA x (Nmax + NA) (the projection on the dual modes) */
        return smat::dense::gemm_ctx_alloc(T.gm, N2, (int)ldF, T.st);
    };
    Transfer T;
    RC(setup(T));
    /* the backward pass on a state, stream and host thread of its own, so
     * that the two directions' latency-bound panel factorisations (a cluster
     * of 16 SMs) run beside each other's products; if the second state does
     * not fit the device, the passes run one after the other on the first */
    Transfer T2;
    const bool concurrent = both_ways && setup(T2) == SMAT_OK;
    if (both_ways && !concurrent) smat_clear_error();
    const size_t lstride = (size_t)2 * 6 * NA1;
    std::vector<const double *> up(nlayers), down(nlayers);
    for (int l = 0; l < nlayers; l++) {
        up[l] = meds + lstride * l;
        down[l] = meds + lstride * (nlayers - 1 - l);
    }
    const int N = nB + nT;
    std::vector<std::complex<double>> Sm((size_t)N * N, 0.0), F01h, B01h, F01b, B01b;
    int rc_back = SMAT_OK;
    std::string msg_back;
    std::thread back;
    if (concurrent) {
        int dev = 0;
        SCK(cudaGetDevice(&dev));
        back = std::thread([&, dev] {
            cudaSetDevice(dev);
            rc_back = one_way(T2, -1, nlayers, down.data(), omega, XiT, XiB, nT, nB, F01b, B01b);
            if (rc_back) msg_back = smat_last_error();
        });
    }
    /* forward: Smat_calc :148-158 */
    const int rc_fwd = one_way(T, 1, nlayers, up.data(), omega, XiB, XiT, nB, nT, F01h, B01h);
    if (back.joinable()) back.join();
    RC(rc_fwd);
    if (rc_back) return smat_fail(rc_back, "%s", msg_back.c_str());
    for (int c = 0; c < N; c++)
        for (int r = 0; r < N; r++)
            Sm[r + (size_t)N * c] = c < nB ? F01h[r + (size_t)N * c] : B01h[r + (size_t)N * (c - nB)];
    if (both_ways) { /* backward: Smat_calc :159-168 */
        if (!concurrent) RC(one_way(T, -1, nlayers, down.data(), omega, XiT, XiB, nT, nB, F01b, B01b));
        for (int c = nB; c < N; c++) {
            for (int r = nB; r < N; r++) Sm[r + (size_t)N * c] = F01b[(r - nB) + (size_t)N * (c - nB)];
            for (int r = 0; r < nB; r++) Sm[r + (size_t)N * c] = F01b[(r + nT) + (size_t)N * (c - nB)];
        }
    }
    if (concurrent) {
        int hinfo2 = 0;
        SCK(cudaMemcpyAsync(&hinfo2, T2.dinfo, sizeof(int), cudaMemcpyDeviceToHost, T2.st));
        SCK(cudaStreamSynchronize(T2.st));
        RC(smat::dense::gemm_ctx_check(T2.gm));
        if (hinfo2 != 0) return smat_fail(SMAT_ENUMERIC, "smat_scalc: singular matrix in the layer transfer (zgesv info)");
        T.solves += T2.solves;
    }
    int hinfo = 0;
    SCK(cudaMemcpyAsync(&hinfo, T.dinfo, sizeof(int), cudaMemcpyDeviceToHost, T.st));
    SCK(cudaStreamSynchronize(T.st));
    RC(smat::dense::gemm_ctx_check(T.gm));
    if (hinfo != 0) return smat_fail(SMAT_ENUMERIC, "smat_scalc: singular matrix in the layer transfer (zgesv info)");
    std::memcpy(S, Sm.data(), sizeof(double2) * Sm.size());
    if (info) {
        /* check_Smat :885-912 */
        double u = 0.0, t = 0.0;
        for (int c = 0; c < N; c++)
            for (int r = 0; r < N; r++) {
                std::complex<double> acc = 0.0;
                for (int k = 0; k < N; k++) acc += std::conj(Sm[k + (size_t)N * r]) * Sm[k + (size_t)N * c];
                if (r == c) acc -= 1.0;
                u += std::norm(acc);
                t += std::norm(Sm[r + (size_t)N * c] - Sm[c + (size_t)N * r]);
            }
        info->unitarity = std::sqrt(u);
        info->transpose = std::sqrt(t);
        info->solves = T.solves;
        info->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return SMAT_OK;
}
