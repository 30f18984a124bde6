/*
 * FP64 split-field FDTD step, bit-identical to the reference main_calc
 * (FDTDcalc/FDTDsplitfieldMetal.c:242-329).
 *
 * One thread per cell and excitation.  Every floating-point expression keeps
 * the reference's operands and order, and the file is compiled with
 * -fmad=false so that no multiply-add is fused: each result is the same IEEE
 * double the reference computes.  The two sweeps have no intra-sweep
 * dependence (the H sweep reads only E, the E sweep only H), so the
 * reference's sequential cell order does not matter.
 *
 * Deliberate differences that change no value: the boundary factor iBc in
 * {-1, 0, 1} multiplies by sign manipulation instead of a DMUL (bp*x for
 * finite x); an ordinary cell with no special neighbour skips the curl of the
 * aux arrays, which the reference evaluates as a sum of zeros; the 0.0 the
 * reference starts each curl sum from is dropped.  These can only flip the
 * sign of a zero.
 */
#include <cuda_runtime.h>

#include "fdtd_internal.cuh"

namespace smat {

/* bp*x for bp in {-1, 0, 1}: keep/flip masks on the bit pattern */
struct Sel {
    unsigned long long keep, flip;
};

__device__ __forceinline__ Sel make_sel(int bc, bool at_edge)
{
    Sel s{~0ull, 0ull};
    if (at_edge) {
        if (bc == 0) s.keep = 0x8000000000000000ull; /* 0*x = zero with the sign of x */
        else if (bc < 0) s.flip = 0x8000000000000000ull;
    }
    return s;
}

__device__ __forceinline__ double bmul(double x, Sel s)
{
    return __longlong_as_double((long long)((((unsigned long long)__double_as_longlong(x)) & s.keep) ^ s.flip));
}

struct Stn {
    long long o[3]; /* offset of the neighbour along each axis (wrapped) */
    Sel s[3];       /* its boundary factor */
};

/* neighbours of ope_R (forward, :374-381) or ope_Rd (backward, :395-402) */
__device__ __forceinline__ Stn make_stn(const Geo &g, int j0, int j1, int j2, bool fwd)
{
    Stn st;
    const int j[3] = {j0, j1, j2};
    const int L[3] = {g.L0, g.L1, g.L2};
    long long stride = 1;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const bool edge = fwd ? (j[a] + 1 == L[a]) : (j[a] == 0);
        const int jn = fwd ? (edge ? 0 : j[a] + 1) : (edge ? L[a] - 1 : j[a] - 1);
        st.o[a] = (long long)(jn - j[a]) * stride;
        st.s[a] = make_sel(g.bc[a], edge);
        stride *= L[a];
    }
    return st;
}

/* Half curls of the main array F ([3][n3]) at cell l.  pl[c]: the term
 * differentiated along axis c+1 ("+" half), mi[c]: along axis c+2. */
template <bool FWD>
__device__ __forceinline__ void curl_main(const double *__restrict__ F, long long n3, long long l,
                                          const Stn &st, double pl[3], double mi[3])
{
    const double h0 = F[l], h1 = F[n3 + l], h2 = F[2 * n3 + l];
    const double here[3] = {h0, h1, h2};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        const double n2 = bmul(F[a2 * n3 + l + st.o[a1]], st.s[a1]);
        const double n1 = bmul(F[a1 * n3 + l + st.o[a2]], st.s[a2]);
        if (!FWD) {
            pl[c] = here[a2] - n2; /* +E - Bp*E(j-1)   (:407) */
            mi[c] = -here[a1] + n1; /* -E + Bp*E(j-1)  (:410) */
        } else {
            pl[c] = n2 - here[a2]; /* +Bp*H(j+1) - H   (:386) */
            mi[c] = -n1 + here[a1]; /* -Bp*H(j+1) + H  (:389) */
        }
    }
}

/* The same on the aux arrays through address_notn (ope_Rmap :330-350,
 * ope_Rdmap :351-371); Fa is [3][lnotn+1] with a zero sentinel. */
template <bool FWD>
__device__ __forceinline__ void curl_aux(const double *__restrict__ Fa, long long as, const int *__restrict__ addr,
                                         long long l, const Stn &st, double pl[3], double mi[3])
{
    const int ah = addr[l];
    const int an[3] = {addr[l + st.o[0]], addr[l + st.o[1]], addr[l + st.o[2]]};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        const double here2 = Fa[a2 * as + ah], here1 = Fa[a1 * as + ah];
        const double n2 = bmul(Fa[a2 * as + an[a1]], st.s[a1]);
        const double n1 = bmul(Fa[a1 * as + an[a2]], st.s[a2]);
        if (!FWD) {
            pl[c] = here2 - n2;
            mi[c] = -here1 + n1;
        } else {
            pl[c] = n2 - here2;
            mi[c] = -n1 + here1;
        }
    }
}

/* Sheet source value of component v at pixel p (main :155-157 or explicit). */
__device__ __forceinline__ double sheet(const Src &s, int pl, int b, int k, bool efield, int v, int p)
{
    if (s.xsrc) return s.xsrc[(efield ? 2 * pl : 0) + v + 2 * p];
    const double *sc = s.sched + 6 * (long long)k + (efield ? 0 : 3);
    const double *w = s.inc + (long long)b * 8 * pl + (efield ? 4 * pl : 0) + 2 * (v + 2 * p);
    const double t = sc[1] * w[0] - (-sc[2]) * w[1]; /* creal(conj(ExpN)*inc) */
    return sc[0] * t;                                /* (2*env) * ... */
}

/* H sweep, main_calc :255-286 */
__global__ void __launch_bounds__(128) k_h64(const P64 p, const int rel)
{
    const int j0 = blockIdx.x * 32 + threadIdx.x, j1 = blockIdx.y * 4 + threadIdx.y, j2 = blockIdx.z;
    const Geo &g = p.g;
    if (j0 >= g.L0 || j1 >= g.L1) return;
    const long long n3 = g.n3, l = j0 + (long long)g.L0 * (j1 + (long long)g.L1 * j2);
    const uint8_t fl = p.flags[l];
    const int cls = fl & 7;
    if (cls == CLS_E) return; /* the H of an 'e' cell is never updated */
    const Stn st = make_stn(g, j0, j1, j2, false);
    const int k = *p.s.base + rel;
    const long long as = p.lnotn + 1;
    const double *Ah = p.cm, *Bh = p.cm + 3 * n3;
    const double *Aha = p.ca, *Bha = p.ca + 3 * (long long)p.lnotn;
    for (int b = 0; b < p.batch; b++) {
        double *__restrict__ H = p.H + (long long)b * 3 * n3;
        const double *__restrict__ E = p.E + (long long)b * 3 * n3;
        double *__restrict__ Ha = p.Ha + (long long)b * 3 * as;
        const double *__restrict__ Ea = p.Ea + (long long)b * 3 * as;
        double pl[3], mi[3];
        curl_main<false>(E, n3, l, st, pl, mi);
        if (cls == CLS_N) {
            double W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
            if (j2 == p.s.iI[b]) {
                const int px = j0 + g.L0 * j1;
                W[0] += p.s.sgn[b] * sheet(p.s, g.pl, b, k, true, 1, px);
                W[1] -= p.s.sgn[b] * sheet(p.s, g.pl, b, k, true, 0, px);
            }
            double h[3];
#pragma unroll
            for (int c = 0; c < 3; c++) h[c] = Ah[c * n3 + l] * H[c * n3 + l] + Bh[c * n3 + l] * (-W[c]);
            if (fl & FL_BWD) {
                double pa[3], ma[3];
                curl_aux<false>(Ea, as, p.addr, l, st, pa, ma);
#pragma unroll
                for (int c = 0; c < 3; c++) h[c] += Bh[c * n3 + l] * (-(pa[c] + ma[c]));
            }
#pragma unroll
            for (int c = 0; c < 3; c++) H[c * n3 + l] = h[c];
        } else if (cls == CLS_A) {
            double pa[3], ma[3];
            curl_aux<false>(Ea, as, p.addr, l, st, pa, ma);
            const int a = p.addr[l];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                double h = Ah[c * n3 + l] * H[c * n3 + l] + Bh[c * n3 + l] * (-pl[c]);
                h += Bh[c * n3 + l] * (-pa[c]);
                H[c * n3 + l] = h;
                double x = Aha[c * p.lnotn + a] * Ha[c * as + a] + Bha[c * p.lnotn + a] * (-mi[c]);
                x += Bha[c * p.lnotn + a] * (-ma[c]);
                Ha[c * as + a] = x;
            }
        } else { /* 'h' or 'b': stable form, main-array curl only (:277-283) */
            const int a = p.addr[l];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double W = pl[c] + mi[c];
                double h = H[c * n3 + l];
                double x = Ha[c * as + a];
                h += 0.5 * x;
                x = Aha[c * p.lnotn + a] * x + Bha[c * p.lnotn + a] * (-W);
                h += 0.5 * x;
                Ha[c * as + a] = x;
                H[c * n3 + l] = h;
            }
        }
    }
}

/* E sweep, main_calc :287-317 */
__global__ void __launch_bounds__(128) k_e64(const P64 p, const int rel)
{
    const int j0 = blockIdx.x * 32 + threadIdx.x, j1 = blockIdx.y * 4 + threadIdx.y, j2 = blockIdx.z;
    const Geo &g = p.g;
    if (j0 >= g.L0 || j1 >= g.L1) return;
    const long long n3 = g.n3, l = j0 + (long long)g.L0 * (j1 + (long long)g.L1 * j2);
    const uint8_t fl = p.flags[l];
    const int cls = fl & 7;
    if (cls == CLS_H) return; /* the E of an 'h' cell is never updated */
    const bool stable = (cls == CLS_E || cls == CLS_B);
    /* the stable form takes the BACKWARD difference of H (:310) */
    const Stn st = make_stn(g, j0, j1, j2, !stable);
    const int k = *p.s.base + rel;
    const long long as = p.lnotn + 1;
    const double *Ae = p.cm + 6 * n3, *Be = p.cm + 9 * n3;
    const double *Aea = p.ca + 6 * (long long)p.lnotn, *Bea = p.ca + 9 * (long long)p.lnotn;
    for (int b = 0; b < p.batch; b++) {
        double *__restrict__ E = p.E + (long long)b * 3 * n3;
        const double *__restrict__ H = p.H + (long long)b * 3 * n3;
        double *__restrict__ Ea = p.Ea + (long long)b * 3 * as;
        const double *__restrict__ Ha = p.Ha + (long long)b * 3 * as;
        double pl[3], mi[3];
        if (stable) {
            curl_main<false>(H, n3, l, st, pl, mi);
            const int a = p.addr[l];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double W = pl[c] + mi[c];
                double e = E[c * n3 + l];
                double x = Ea[c * as + a];
                e += 0.5 * x;
                x = Aea[c * p.lnotn + a] * x + Bea[c * p.lnotn + a] * W;
                e += 0.5 * x;
                Ea[c * as + a] = x;
                E[c * n3 + l] = e;
            }
            continue;
        }
        curl_main<true>(H, n3, l, st, pl, mi);
        if (cls == CLS_N) {
            double W[3] = {pl[0] + mi[0], pl[1] + mi[1], pl[2] + mi[2]};
            if (j2 == p.s.iI[b]) {
                const int px = j0 + g.L0 * j1;
                W[0] += p.s.sgn[b] * sheet(p.s, g.pl, b, k, false, 1, px);
                W[1] -= p.s.sgn[b] * sheet(p.s, g.pl, b, k, false, 0, px);
            }
            double e[3];
#pragma unroll
            for (int c = 0; c < 3; c++) e[c] = Ae[c * n3 + l] * E[c * n3 + l] + Be[c * n3 + l] * W[c];
            if (fl & FL_FWD) {
                double pa[3], ma[3];
                curl_aux<true>(Ha, as, p.addr, l, st, pa, ma);
#pragma unroll
                for (int c = 0; c < 3; c++) e[c] += Be[c * n3 + l] * (pa[c] + ma[c]);
            }
#pragma unroll
            for (int c = 0; c < 3; c++) E[c * n3 + l] = e[c];
        } else { /* 'a' */
            double pa[3], ma[3];
            curl_aux<true>(Ha, as, p.addr, l, st, pa, ma);
            const int a = p.addr[l];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                double e = Ae[c * n3 + l] * E[c * n3 + l] + Be[c * n3 + l] * pl[c];
                e += Be[c * n3 + l] * pa[c];
                E[c * n3 + l] = e;
                double x = Aea[c * p.lnotn + a] * Ea[c * as + a] + Bea[c * p.lnotn + a] * mi[c];
                x += Bea[c * p.lnotn + a] * ma[c];
                Ea[c * as + a] = x;
            }
        }
    }
}

/* running DFT on the monitor planes (main_calc :318-328), FP64 accumulators.
 * acc += phase * x computed as (re += pr*x, im += pi*x), the value of the
 * reference's complex product with a real factor. */
__global__ void k_dft64(const P64 p, const int rel)
{
    const int px = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y, b = blockIdx.z;
    const Geo &g = p.g;
    if (px >= g.pl) return;
    const long long n3 = g.n3, off = (long long)p.d.planes[q] * g.pl + px;
    const double *H = p.H + (long long)b * 3 * n3, *E = p.E + (long long)b * 3 * n3;
    double x[4] = {H[off], H[n3 + off], E[off], E[n3 + off]};
    if ((p.flags[off] & 7) == CLS_A) {
        /* a plane through the PML (allowed for general schedules only; the
         * reference exits, :320): sample the total field main + aux */
        const long long as = p.lnotn + 1, a = p.addr[off];
        const double *Ha = p.Ha + (long long)b * 3 * as, *Ea = p.Ea + (long long)b * 3 * as;
        x[0] += Ha[a];
        x[1] += Ha[as + a];
        x[2] += Ea[a];
        x[3] += Ea[as + a];
    }
    const int k = *p.s.base + rel;
    for (int f = 0; f < p.d.nfreq; f++) {
        const double *ph = p.d.xphase ? p.d.xphase : p.d.phase + 4 * ((long long)k * p.d.nfreq + f);
        double *acc = p.d.acc + 2 * ((((long long)b * p.d.nfreq + f) * p.d.nq + q) * 4 * g.pl + px);
#pragma unroll
        for (int v = 0; v < 4; v++) {
            const double pr = ph[v < 2 ? 0 : 2], pi = ph[v < 2 ? 1 : 3];
            double *a = acc + 2 * (long long)v * g.pl;
            a[0] += pr * x[v];
            a[1] += pi * x[v];
        }
    }
}

__global__ void k_bump(int *base, int by)
{
    *base += by;
}

__global__ void k_set(int *base, int value)
{
    *base = value;
}

/* max |x| as the bit pattern of a non-negative double (NaN sorts above Inf) */
__global__ void k_maxabs(const void *x, long long n, int is_double, unsigned long long *out)
{
    unsigned long long m = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = is_double ? ((const double *)x)[i] : (double)((const float *)x)[i];
        const unsigned long long bits = (unsigned long long)__double_as_longlong(fabs(v));
        m = bits > m ? bits : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_down_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

void launch_h64(const P64 &p, int rel, cudaStream_t st)
{
    dim3 blk(32, 4, 1), grd((p.g.L0 + 31) / 32, (p.g.L1 + 3) / 4, p.g.L2);
    k_h64<<<grd, blk, 0, st>>>(p, rel);
}

void launch_e64(const P64 &p, int rel, cudaStream_t st)
{
    dim3 blk(32, 4, 1), grd((p.g.L0 + 31) / 32, (p.g.L1 + 3) / 4, p.g.L2);
    k_e64<<<grd, blk, 0, st>>>(p, rel);
}

void launch_dft64(const P64 &p, int rel, cudaStream_t st)
{
    if (p.d.nfreq <= 0 || p.d.nq <= 0) return;
    dim3 blk(256), grd((p.g.pl + 255) / 256, p.d.nq, p.batch);
    k_dft64<<<grd, blk, 0, st>>>(p, rel);
}

void launch_bump(int *base, int by, cudaStream_t st) { k_bump<<<1, 1, 0, st>>>(base, by); }

void launch_set(int *base, int value, cudaStream_t st) { k_set<<<1, 1, 0, st>>>(base, value); }

void launch_maxabs(const void *x, long long n, int is_double, double *out, cudaStream_t st)
{
    k_maxabs<<<608, 256, 0, st>>>(x, n, is_double, (unsigned long long *)out);
}

} // namespace smat
