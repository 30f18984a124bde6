/*
 * Host precompute of the split-field FDTD: the FP64 set-up the reference does
 * before its time loop (FDTDcalc/FDTDsplitfieldMetal.c main :62-143).
 *
 * Compiled as C11 with -O2 -ffp-contract=off (the reference's own flags plus
 * no FMA contraction) and written with the reference's operand order in every
 * floating-point expression, so coefficients, envelopes and phases are
 * bit-identical to the reference's on the same host.  That is what lets the
 * FP64 GPU path reproduce the reference's fields exactly.
 */
#define _POSIX_C_SOURCE 200809L /* sysconf under -std=c11 */

#include "smatran_fdtd.h"
#include "host_internal.h"

#include <complex.h>
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define TWO_PI_LD (2.0L * 3.1415926535897932384626433832795028841971L) /* constant.h:13-15 */
#define TINY (10.0 * DBL_EPSILON)                                      /* constant.h:7 */

static int dims_ok(const int L[4])
{
    return L && L[0] > 0 && L[1] > 0 && L[2] > 0 && L[3] >= 0 &&
           (long long)L[0] * L[1] * L[2] < (1LL << 31) / 3;
}

/* ---- sigma from the stretched media: set_sigma :858-926 ---------------- */

int smat_set_sigma(const int L[4], const double *mu_, const double *epsi_, double *sigma)
{
    if (!dims_ok(L) || !mu_ || !epsi_ || !sigma) return smat_fail(SMAT_EINVAL, "set_sigma: bad arguments");
    const double complex *mu = (const double complex *)mu_;
    const double complex *ep = (const double complex *)epsi_;
    const int L0 = L[0], L1 = L[1], L2 = L[2];
    const long s1 = L0, s2 = (long)L0 * L1;
    memset(sigma, 0, sizeof(double) * 2 * (L0 + L1 + L2));
    /* For axis a the H-half value comes from arg(mu_{a+1}), arg(mu_{a+2}) and
     * -arg(epsi_a) on the centre line along a; the E half swaps mu and epsi.
     * The three must agree to 10*DBL_EPSILON; sigma = tan() of the one the
     * reference labels 00. */
    /* axis 0, line (j1, j2) = (L1/2, L2/2) */
    for (int j = 0; j < L0; j++) {
        const long b = 3 * (j + s1 * (L1 / 2) + s2 * (L2 / 2));
        for (int h = 0; h < 2; h++) {
            const double complex *P = h ? ep : mu, *Q = h ? mu : ep;
            const double a11 = carg(P[b + 1]);
            if (a11 == 0.) continue;
            const double a22 = carg(P[b + 2]);
            const double a00 = -carg(Q[b + 0]);
            if (fabs(a00 - a11) < TINY && fabs(a11 - a22) < TINY && fabs(a22 - a00) < TINY)
                sigma[h + 2 * j] = tan(a00);
        }
    }
    /* axis 1, line (j0, j2) = (L0/2, L2/2) */
    for (int j = 0; j < L1; j++) {
        const long b = 3 * ((L0 / 2) + s1 * j + s2 * (L2 / 2));
        for (int h = 0; h < 2; h++) {
            const double complex *P = h ? ep : mu, *Q = h ? mu : ep;
            const double a22 = carg(P[b + 2]);
            if (a22 == 0.) continue;
            const double a00 = carg(P[b + 0]);
            const double a11 = -carg(Q[b + 1]);
            if (fabs(a00 - a11) < TINY && fabs(a11 - a22) < TINY && fabs(a22 - a00) < TINY)
                sigma[2 * L0 + h + 2 * j] = tan(a00);
        }
    }
    /* axis 2, line (j0, j1) = (L0/2, L1/2) */
    for (int j = 0; j < L2; j++) {
        const long b = 3 * ((L0 / 2) + s1 * (L1 / 2) + s2 * j);
        for (int h = 0; h < 2; h++) {
            const double complex *P = h ? ep : mu, *Q = h ? mu : ep;
            const double a00 = carg(P[b + 0]);
            if (a00 == 0.) continue;
            const double a11 = carg(P[b + 1]);
            const double a22 = -carg(Q[b + 2]);
            if (fabs(a00 - a11) < TINY && fabs(a11 - a22) < TINY && fabs(a22 - a00) < TINY)
                sigma[2 * L0 + 2 * L1 + h + 2 * j] = tan(a00);
        }
    }
    return SMAT_OK;
}

/* ---- remove_sigma :822-853 ---------------------------------------------- */

/* 1 + i*sigma for every (axis, index, half): the stretch s_j of the reference */
static double complex *axis_stretch(const int L[4], const double *sigma)
{
    const int n = 2 * (L[0] + L[1] + L[2]);
    double complex *s = malloc(sizeof(double complex) * n);
    if (!s) return NULL;
    for (int i = 0; i < n; i++) s[i] = 1. + I * sigma[i];
    return s;
}

int smat_remove_sigma(const int L[4], double *mu_, double *epsi_, const double *sigma)
{
    if (!dims_ok(L) || !mu_ || !epsi_ || !sigma) return smat_fail(SMAT_EINVAL, "remove_sigma: bad arguments");
    double complex *s = axis_stretch(L, sigma);
    if (!s) return smat_fail(SMAT_ENOMEM, "remove_sigma: out of host memory");
    const int off[3] = {0, 2 * L[0], 2 * (L[0] + L[1])};
    double complex *fld[2] = {(double complex *)mu_, (double complex *)epsi_};
    int rc = SMAT_OK;
    for (int j2 = 0; j2 < L[2] && rc == SMAT_OK; j2++)
        for (int j1 = 0; j1 < L[1] && rc == SMAT_OK; j1++)
            for (int j0 = 0; j0 < L[0] && rc == SMAT_OK; j0++) {
                const int jj[3] = {j0, j1, j2};
                const long l = j0 + (long)L[0] * j1 + (long)L[0] * L[1] * j2;
                for (int which = 0; which < 2; which++) {
                    /* mu: numerator on the H sub-point (h = 0) of the two other axes,
                     * denominator on the E sub-point of its own axis; epsi: swapped */
                    const int hn = which, hd = 1 - which;
                    for (int c = 0; c < 3; c++) {
                        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
                        const double complex sd = s[off[c] + hd + 2 * jj[c]];
                        const double complex cn = s[off[a1] + hn + 2 * jj[a1]] * s[off[a2] + hn + 2 * jj[a2]] *
                                                  conj(sd) / (creal(sd) * creal(sd) + cimag(sd) * cimag(sd));
                        double complex *v = &fld[which][c + 3 * l];
                        *v *= conj(cn) / (creal(cn) * creal(cn) + cimag(cn) * cimag(cn));
                        if (cimag(cn) != 0.) {
                            if (fabs(carg(*v)) > TINY) {
                                rc = smat_fail(SMAT_EINVAL, "remove_sigma: %s at cell %ld is not a stretched real value",
                                               which ? "epsi" : "mu", l);
                                break;
                            }
                            *v = creal(*v);
                        }
                    }
                }
            }
    free(s);
    return rc;
}

/* ---- host worker threads ------------------------------------------------ */

int host_threads(long long work)
{
    const char *e = getenv("SMATRAN_HOST_THREADS");
    if (e && *e) {
        const int n = atoi(e);
        if (n >= 1 && n <= HOST_MAX_THREADS) return n;
    }
    if (work < (1LL << 20)) return 1;
    const long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c < 1 ? 1 : c < 16 ? (int)c : 16;
}

struct host_range {
    host_range_fn fn;
    void *ctx;
    long long lo, hi;
};

static void *host_range_main(void *a)
{
    const struct host_range *r = (const struct host_range *)a;
    r->fn(r->ctx, r->lo, r->hi);
    return NULL;
}

void host_parallel_for(long long n, int nt, host_range_fn fn, void *ctx)
{
    if (nt > HOST_MAX_THREADS) nt = HOST_MAX_THREADS;
    if ((long long)nt > n) nt = (int)n;
    if (nt <= 1) {
        if (n > 0) fn(ctx, 0, n);
        return;
    }
    pthread_t th[HOST_MAX_THREADS];
    struct host_range r[HOST_MAX_THREADS];
    int started[HOST_MAX_THREADS];
    for (int t = 0; t < nt; t++) {
        r[t].fn = fn;
        r[t].ctx = ctx;
        r[t].lo = n * t / nt;
        r[t].hi = n * (t + 1) / nt;
        started[t] = t > 0 && pthread_create(&th[t], NULL, host_range_main, &r[t]) == 0;
    }
    host_range_main(&r[0]);
    /* a range whose thread could not be created runs here */
    for (int t = 1; t < nt; t++)
        if (started[t]) pthread_join(th[t], NULL);
        else host_range_main(&r[t]);
}

/* ---- set_address :188-233 ---------------------------------------------- */

struct address_job {
    const int *L;
    const double complex *mu, *ep;
    const unsigned char *pml[3];
    char *Cont;
    int *address_notn;
    int nrun;
    int *count; /* [nrun]: non-'n' cells of each run, then the first address of each */
    int total;
};

/* run t: planes [z0, z1) */
static void address_run(const struct address_job *J, long long t, int *z0, int *z1)
{
    *z0 = (int)(J->L[2] * t / J->nrun);
    *z1 = (int)(J->L[2] * (t + 1) / J->nrun);
}

/* classify the cells of runs [t0, t1) and count the split ones */
static void address_classify(void *ctx, long long t0, long long t1)
{
    struct address_job *J = (struct address_job *)ctx;
    const int *L = J->L;
    for (long long t = t0; t < t1; t++) {
        int z0, z1;
        address_run(J, t, &z0, &z1);
        long l = (long)z0 * L[0] * L[1];
        int count = 0;
        for (int j2 = z0; j2 < z1; j2++)
            for (int j1 = 0; j1 < L[1]; j1++)
                for (int j0 = 0; j0 < L[0]; j0++, l++) {
                    char k = (J->pml[0][j0] || J->pml[1][j1] || J->pml[2][j2]) ? 'a' : 'n';
                    /* lossy media override, the last component deciding (:200-210) */
                    for (int c = 0; c < 3; c++) {
                        /* with a zero imaginary part tan(carg()) is 0 or +-1.2e-16,
                         * never below -TINY: skip the trigonometry (same answer) */
                        const int m = cimag(J->mu[c + 3 * l]) != 0.0 && tan(carg(J->mu[c + 3 * l])) < -TINY;
                        const int e = cimag(J->ep[c + 3 * l]) != 0.0 && tan(carg(J->ep[c + 3 * l])) < -TINY;
                        if (m && e) k = 'b';
                        else if (m) k = 'h';
                        else if (e) k = 'e';
                    }
                    J->Cont[l] = k;
                    if (k != 'n') count++;
                }
        J->count[t] = count;
    }
}

/* addresses in cell order: a run starts at the split cells of the runs before it */
static void address_number(void *ctx, long long t0, long long t1)
{
    struct address_job *J = (struct address_job *)ctx;
    for (long long t = t0; t < t1; t++) {
        int z0, z1;
        address_run(J, t, &z0, &z1);
        const long pl = (long)J->L[0] * J->L[1];
        int next = J->count[t];
        for (long l = z0 * pl; l < z1 * pl; l++) J->address_notn[l] = J->Cont[l] != 'n' ? next++ : J->total;
    }
}

int smat_set_address(const int L[4], const double *sigma, const double *mu_, const double *epsi_,
                     char *Cont, int *Lnotn, int *address_notn)
{
    if (!dims_ok(L) || !sigma || !mu_ || !epsi_ || !Cont || !Lnotn || !address_notn)
        return smat_fail(SMAT_EINVAL, "set_address: bad arguments");
    const int off[3] = {0, 2 * L[0], 2 * (L[0] + L[1])};
    const long n3 = (long)L[0] * L[1] * L[2];
    /* a cell is split ('a') when any of its six sub-point sigmas is nonzero */
    unsigned char *pml[3];
    for (int a = 0; a < 3; a++) {
        pml[a] = malloc(L[a]);
        if (!pml[a]) {
            for (int b = 0; b < a; b++) free(pml[b]);
            return smat_fail(SMAT_ENOMEM, "set_address: out of host memory");
        }
        for (int j = 0; j < L[a]; j++)
            pml[a][j] = fabs(sigma[off[a] + 2 * j]) > TINY || fabs(sigma[off[a] + 1 + 2 * j]) > TINY;
    }
    struct address_job J;
    J.L = L;
    J.mu = (const double complex *)mu_;
    J.ep = (const double complex *)epsi_;
    for (int a = 0; a < 3; a++) J.pml[a] = pml[a];
    J.Cont = Cont;
    J.address_notn = address_notn;
    J.nrun = host_threads(n3);
    if (J.nrun > L[2]) J.nrun = L[2];
    int count[HOST_MAX_THREADS];
    J.count = count;
    host_parallel_for(J.nrun, J.nrun, address_classify, &J);
    J.total = 0;
    for (int t = 0; t < J.nrun; t++) {
        const int c = count[t];
        count[t] = J.total;
        J.total += c;
    }
    host_parallel_for(J.nrun, J.nrun, address_number, &J);
    for (int a = 0; a < 3; a++) free(pml[a]);
    *Lnotn = J.total;
    return SMAT_OK;
}

/* ---- coefficients, main :106-143 ---------------------------------------- */

/* lossless / lossy update factors with stretch sigma (main :118-127) */
static void ab_split(double iR, double iI, double re, double im, double sg, double *A, double *B)
{
    *B = 1. / (iR * re + iI * (re * sg + im));
    *A = (iR * re - iI * (re * sg + im)) * *B;
}

/* the stable form for media with tan(arg) < 0 (StableForm, main :129-139) */
static void ab_stable(double iR, double iI, double re, double im, double *A, double *B)
{
    *B = 1. / (0.5 * re - iR * (0.5 * im / iI));
    *A = -(0.5 * re + iR * (0.5 * im / iI)) * *B;
}

struct coeff_job {
    const int *L;
    long n3;
    size_t len; /* doubles per output array */
    const double *sigma;
    const double complex *mu, *ep;
    const char *Cont;
    const int *address_notn;
    double iR, iI;
    double *Ah, *Bh, *Ae, *Be;
};

static void coeff_zero(void *ctx, long long lo, long long hi)
{
    const struct coeff_job *j = (const struct coeff_job *)ctx;
    double *out[4] = {j->Ah, j->Bh, j->Ae, j->Be};
    for (int w = 0; w < 4; w++) memset(out[w] + lo, 0, sizeof(double) * (size_t)(hi - lo));
}

/* the cells of planes [z0, z1): every cell writes its own three main entries
 * and the aux entries of its own address */
static void coeff_planes(void *ctx, long long z0, long long z1)
{
    const struct coeff_job *J = (const struct coeff_job *)ctx;
    const int *L = J->L;
    const long n3 = J->n3;
    const double iR = J->iR, iI = J->iI;
    const double *sigma = J->sigma;
    double *Ah = J->Ah, *Bh = J->Bh, *Ae = J->Ae, *Be = J->Be;
    const int off[3] = {0, 2 * L[0], 2 * (L[0] + L[1])};
    long l = (long)z0 * L[0] * L[1];
    for (int j2 = (int)z0; j2 < (int)z1; j2++)
        for (int j1 = 0; j1 < L[1]; j1++)
            for (int j0 = 0; j0 < L[0]; j0++, l++) {
                const int jj[3] = {j0, j1, j2};
                const char k = J->Cont[l];
                for (int c = 0; c < 3; c++) {
                    const long m = c + 3 * l;
                    const long x = c + 3L * J->address_notn[l] + 3 * n3;
                    const double mr = creal(J->mu[m]), mi = cimag(J->mu[m]);
                    const double er = creal(J->ep[m]), ei = cimag(J->ep[m]);
                    const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
                    ab_split(iR, iI, mr, mi, sigma[off[a1] + 0 + 2 * jj[a1]], &Ah[m], &Bh[m]);
                    ab_split(iR, iI, er, ei, sigma[off[a1] + 1 + 2 * jj[a1]], &Ae[m], &Be[m]);
                    if (k == 'a') {
                        ab_split(iR, iI, mr, mi, sigma[off[a2] + 0 + 2 * jj[a2]], &Ah[x], &Bh[x]);
                        ab_split(iR, iI, er, ei, sigma[off[a2] + 1 + 2 * jj[a2]], &Ae[x], &Be[x]);
                    }
                    if (k == 'e' || k == 'b') ab_stable(iR, iI, er, ei, &Ae[x], &Be[x]);
                    if (k == 'h' || k == 'b') ab_stable(iR, iI, mr, mi, &Ah[x], &Bh[x]);
                }
            }
}

int smat_coefficients(const int L[4], int Lnotn, const double *sigma, const double *mu_,
                      const double *epsi_, const char *Cont, const int *address_notn,
                      double iR, double iI, double *Ah, double *Bh, double *Ae, double *Be)
{
    if (!dims_ok(L) || Lnotn < 0 || !sigma || !mu_ || !epsi_ || !Cont || !address_notn || !Ah || !Bh ||
        !Ae || !Be)
        return smat_fail(SMAT_EINVAL, "coefficients: bad arguments");
    struct coeff_job J;
    J.L = L;
    J.n3 = (long)L[0] * L[1] * L[2];
    J.len = 3 * (size_t)(J.n3 + Lnotn);
    J.sigma = sigma;
    J.mu = (const double complex *)mu_;
    J.ep = (const double complex *)epsi_;
    J.Cont = Cont;
    J.address_notn = address_notn;
    J.iR = iR;
    J.iI = iI;
    J.Ah = Ah;
    J.Bh = Bh;
    J.Ae = Ae;
    J.Be = Be;
    /* every entry is a pure function of its own cell, so any split of the
     * planes over threads gives the same bits; the zero fill finishes first
     * because a thread's aux entries may lie in another thread's fill range */
    const int nt = host_threads(J.n3);
    host_parallel_for((long long)J.len, nt, coeff_zero, &J);
    host_parallel_for(L[2], nt, coeff_planes, &J);
    return SMAT_OK;
}

/* ---- time parameters ---------------------------------------------------- */

int smat_set_tau(double omega, double min_Dt, int *N_2pi, double *iR, double *iI)
{
    if (!N_2pi || !iR || !iI || !(omega > 0.) || !(min_Dt > 0.))
        return smat_fail(SMAT_EINVAL, "set_tau: omega and min_Dt must be positive");
    int n = 0;
    while (omega * min_Dt * n <= TWO_PI_LD) n++; /* :518 */
    const double dphi = TWO_PI_LD / ((double)n);
    const double dt = dphi / omega;
    *N_2pi = n;
    *iR = (0.5 * dphi) / (dt * sin(0.5 * dphi));
    *iI = (0.5 * omega) / (cos(0.5 * dphi));
    return SMAT_OK;
}

double smat_set_env(int N, const int tp[3], int jh, int jt, int jp)
{
    if (!tp || N <= 0) return NAN;
    const int up = tp[0], flat = tp[0] + tp[1], down = 2 * tp[0] + tp[1];
    double f;
    if (jp < up || (jp >= flat && jp < down)) {
        /* sin^2 ramp-up, cos^2 ramp-down over tp[0] periods (:455-468) */
        const double dphi = TWO_PI_LD / ((double)4 * tp[0]);
        const double dphis = TWO_PI_LD / ((double)4 * tp[0] * N);
        const double complex slow = jp < up ? cexp(I * dphi * ((double)jp))
                                            : cexp(I * dphi * ((double)jp - (tp[0] + tp[1])));
        const double complex fast = cexp(I * dphis * (0.5 * ((double)jh) + ((double)jt)));
        f = jp < up ? cimag(slow * fast) : creal(slow * fast);
    } else if (jp < flat) {
        f = 1.;
    } else if (jp < tp[2]) {
        f = 0.;
    } else {
        return NAN;
    }
    const double norm = 1. / ((double)1 * (tp[0] + tp[1]) * N);
    return norm * f * f;
}

/* exp(i*phi) at whole (2j) and half (2j+1) steps, main :93-99 */
int host_expn(int N, double *out)
{
    double complex *e = (double complex *)out;
    const double dphi = TWO_PI_LD / ((double)N);
    for (int j = 0; j < N; j++) {
        const double p0 = dphi * ((double)j);
        const double p5 = dphi * (0.5 + ((double)j));
        e[2 * j] = cexp(I * p0);
        e[2 * j + 1] = cexp(I * p5);
    }
    return SMAT_OK;
}

/* The reference CW run as a general schedule: for global step k = jp*N + jt,
 * src = {2 env(1,jt,jp), Re, Im of ExpN[1+2jt], 2 env(0,jt+1,jp), Re, Im of
 * ExpN[2((jt+1)%N)]} (main :155-157) and DFT phases {ExpN[2n], ExpN[2n+1]},
 * n = (jt+1)%N (main :165). */
int host_cw_schedule(int N, const int tp[3], double *src, double *phase)
{
    const int nsteps = tp[2] * N;
    double complex *e = malloc(sizeof(double complex) * 2 * N);
    if (!e) return smat_fail(SMAT_ENOMEM, "cw schedule: out of host memory");
    host_expn(N, (double *)e);
    int rc = SMAT_OK;
    for (int k = 0; k < nsteps; k++) {
        const int jp = k / N, jt = k % N, jn = (jt + 1) % N;
        const double sE = (2.) * smat_set_env(N, tp, 1, jt, jp);
        const double sH = (2.) * smat_set_env(N, tp, 0, (jt + 1), jp);
        if (isnan(sE) || isnan(sH)) {
            rc = smat_fail(SMAT_EINVAL, "cw schedule: envelope undefined (stop-period < 2*ramp + cw?)");
            break;
        }
        double *s = src + 6 * (long)k;
        s[0] = sE;
        s[1] = creal(e[1 + 2 * jt]);
        s[2] = cimag(e[1 + 2 * jt]);
        s[3] = sH;
        s[4] = creal(e[2 * jn]);
        s[5] = cimag(e[2 * jn]);
        double *p = phase + 4 * (long)k;
        p[0] = creal(e[2 * jn]);
        p[1] = cimag(e[2 * jn]);
        p[2] = creal(e[2 * jn + 1]);
        p[3] = cimag(e[2 * jn + 1]);
    }
    free(e);
    return rc;
}

/* omega = 2 pi / (lambda k0) as input_Lf evaluates it (:740, long double 2 pi) */
double smat_omega(double wavelength, double k0) { return TWO_PI_LD / (wavelength * k0); }
