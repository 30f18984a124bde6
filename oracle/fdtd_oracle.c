/*
 * CPU oracle for the split-field FDTD time loop -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, function by function, the algorithm of FDTDcalc/FDTDsplitfieldMetal.c
 * (SMatrAnEM).  Every floating-point expression keeps the reference's operand
 * order so that, compiled with -O2 -ffp-contract=off, results agree bit for
 * bit with the reference on the same machine.  The loop structure, helpers and
 * names are this file's own.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load it; the product never does.
 */
#include "fdtd_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* 2*pi in long double, the precision the reference evaluates its phase
 * increments in (FDTDcalc/constant.h:13-15). */
#define ORC_TWO_PI (2.0L * 3.1415926535897932384626433832795028841971L)
/* threshold for "nonzero" sigma and "negative" tan(arg) (FDTDcalc/constant.h:7) */
#define ORC_TINY (10.0 * DBL_EPSILON)

/* ------------------------------------------------------------------------ */
/* sigma recovery: FDTDsplitfieldMetal.c:858-926.
 * The stretch s_j = 1 + i*sigma_j is read back from arg(mu), arg(epsi) on the
 * centre lines of the grid; sigma[2*j0 + h] along axis 0, then axis 1 at offset
 * 2*L0, axis 2 at offset 2*(L0+L1); h = 0 for the H sub-point, 1 for E. */
static int same3(double a, double b, double c)
{
    return fabs(a - b) < ORC_TINY && fabs(b - c) < ORC_TINY && fabs(c - a) < ORC_TINY;
}

void orc_set_sigma(const int L[4], const double complex *mu, const double complex *epsi,
                   double *sigma)
{
    const int L0 = L[0], L1 = L[1], L2 = L[2];
    const int c0 = L0 / 2, c1 = L1 / 2, c2 = L2 / 2;
    /* axis 0 along (j1, j2) = (L1/2, L2/2): :860-881 */
    for (int j0 = 0; j0 < L0; j0++) {
        const long l = 3L * (j0 + (long)L0 * c1 + (long)L0 * L1 * c2);
        double p = carg(mu[l + 1]);
        if (p != 0.) {
            double q = carg(mu[l + 2]), r = -carg(epsi[l + 0]);
            if (same3(r, p, q)) sigma[0 + 2 * j0] = tan(r);
        }
        p = carg(epsi[l + 1]);
        if (p != 0.) {
            double q = carg(epsi[l + 2]), r = -carg(mu[l + 0]);
            if (same3(r, p, q)) sigma[1 + 2 * j0] = tan(r);
        }
    }
    /* axis 1 along (j0, j2) = (L0/2, L2/2): :882-903 */
    for (int j1 = 0; j1 < L1; j1++) {
        const long l = 3L * (c0 + (long)L0 * j1 + (long)L0 * L1 * c2);
        double q = carg(mu[l + 2]);
        if (q != 0.) {
            double r = carg(mu[l + 0]), p = -carg(epsi[l + 1]);
            if (same3(r, p, q)) sigma[2 * L0 + 0 + 2 * j1] = tan(r);
        }
        q = carg(epsi[l + 2]);
        if (q != 0.) {
            double r = carg(epsi[l + 0]), p = -carg(mu[l + 1]);
            if (same3(r, p, q)) sigma[2 * L0 + 1 + 2 * j1] = tan(r);
        }
    }
    /* axis 2 along (j0, j1) = (L0/2, L1/2): :904-925 */
    for (int j2 = 0; j2 < L2; j2++) {
        const long l = 3L * (c0 + (long)L0 * c1 + (long)L0 * L1 * j2);
        double r = carg(mu[l + 0]);
        if (r != 0.) {
            double p = carg(mu[l + 1]), q = -carg(epsi[l + 2]);
            if (same3(r, p, q)) sigma[2 * L0 + 2 * L1 + 0 + 2 * j2] = tan(r);
        }
        r = carg(epsi[l + 0]);
        if (r != 0.) {
            double p = carg(epsi[l + 1]), q = -carg(mu[l + 2]);
            if (same3(r, p, q)) sigma[2 * L0 + 2 * L1 + 1 + 2 * j2] = tan(r);
        }
    }
}

/* per-cell stretch factors s[h + 2*axis] = 1 + i*sigma (remove_sigma :826-830) */
static void cell_stretch(const int L[4], const double *sigma, int j0, int j1, int j2,
                         double complex s[6])
{
    for (int h = 0; h < 2; h++) {
        s[h + 0] = 1. + I * sigma[h + 2 * j0];
        s[h + 2] = 1. + I * sigma[2 * L[0] + h + 2 * j1];
        s[h + 4] = 1. + I * sigma[2 * L[0] + 2 * L[1] + h + 2 * j2];
    }
}

/* divide out s_{c+1} s_{c+2} / s_c from each component: remove_sigma :822-853 */
static int unstretch(double complex *v, const double complex s[6], int hn, int hd)
{
    for (int c = 0; c < 3; c++) {
        const double complex sd = s[hd + 2 * c];
        const double complex cn = s[hn + 2 * ((c + 1) % 3)] * s[hn + 2 * ((c + 2) % 3)] * conj(sd)
                                  / (creal(sd) * creal(sd) + cimag(sd) * cimag(sd));
        v[c] *= conj(cn) / (creal(cn) * creal(cn) + cimag(cn) * cimag(cn));
        if (cimag(cn) != 0.) {
            if (fabs(carg(v[c])) > ORC_TINY) return -1;
            v[c] = creal(v[c]);
        }
    }
    return 0;
}

int orc_remove_sigma(const int L[4], double complex *mu, double complex *epsi,
                     const double *sigma)
{
    for (int j2 = 0; j2 < L[2]; j2++)
        for (int j1 = 0; j1 < L[1]; j1++)
            for (int j0 = 0; j0 < L[0]; j0++) {
                const long l = 3L * (j0 + (long)L[0] * j1 + (long)L[0] * L[1] * j2);
                double complex s[6];
                cell_stretch(L, sigma, j0, j1, j2, s);
                /* mu: numerator at the H sub-point (h=0), denominator at E (h=1) */
                if (unstretch(&mu[l], s, 0, 1)) return -1;
                if (unstretch(&epsi[l], s, 1, 0)) return -1;
            }
    return 0;
}

/* sigma6[h + 2*axis] of a cell, the layout the coefficient formulas index */
static void cell_sigma6(const int L[4], const double *sigma, int j0, int j1, int j2, double s6[6])
{
    for (int h = 0; h < 2; h++) {
        s6[h + 0] = sigma[h + 2 * j0];
        s6[h + 2] = sigma[2 * L[0] + h + 2 * j1];
        s6[h + 4] = sigma[2 * L[0] + 2 * L[1] + h + 2 * j2];
    }
}

/* ------------------------------------------------------------------------ */
/* cell classes: set_address :188-233 */
int orc_set_address(const int L[4], const double *sigma, const double complex *mu,
                    const double complex *epsi, char *Cont, int *address_notn)
{
    const long n3 = (long)L[0] * L[1] * L[2];
    for (int j2 = 0; j2 < L[2]; j2++)
        for (int j1 = 0; j1 < L[1]; j1++)
            for (int j0 = 0; j0 < L[0]; j0++) {
                const long l = j0 + (long)L[0] * j1 + (long)L[0] * L[1] * j2;
                double s6[6];
                cell_sigma6(L, sigma, j0, j1, j2, s6);
                char k = 'n';
                for (int i = 0; i < 6; i++)
                    if (fabs(s6[i]) > ORC_TINY) k = 'a';
                for (int c = 0; c < 3; c++) {
                    const int lossy_mu = tan(carg(mu[c + 3 * l])) < -ORC_TINY;
                    const int lossy_ep = tan(carg(epsi[c + 3 * l])) < -ORC_TINY;
                    if (lossy_mu && lossy_ep) k = 'b';
                    else if (lossy_mu) k = 'h';
                    else if (lossy_ep) k = 'e';
                }
                Cont[l] = k;
            }
    int nspecial = 0;
    for (long l = 0; l < n3; l++)
        if (Cont[l] != 'n') nspecial++;
    int next = 0;
    for (long l = 0; l < n3; l++)
        address_notn[l] = (Cont[l] != 'n') ? next++ : nspecial;
    return nspecial;
}

/* ------------------------------------------------------------------------ */
/* update coefficients: main :106-143 and StableForm for lossy cells */
void orc_coefficients(const int L[4], int Lnotn, const double *sigma,
                      const double complex *mu, const double complex *epsi,
                      const char *Cont, const int *address_notn,
                      double invtau_R, double invtau_I,
                      double *Ah, double *Bh, double *Ae, double *Be)
{
    (void)Lnotn;
    const long n3 = (long)L[0] * L[1] * L[2];
    for (int j2 = 0; j2 < L[2]; j2++)
        for (int j1 = 0; j1 < L[1]; j1++)
            for (int j0 = 0; j0 < L[0]; j0++) {
                const long l = j0 + (long)L[0] * j1 + (long)L[0] * L[1] * j2;
                double s6[6];
                cell_sigma6(L, sigma, j0, j1, j2, s6);
                for (int c = 0; c < 3; c++) {
                    const long m = c + 3 * l;
                    const double mr = creal(mu[m]), mi = cimag(mu[m]);
                    const double er = creal(epsi[m]), ei = cimag(epsi[m]);
                    /* main slot: the half driven along axis c+1 */
                    double sh = s6[0 + 2 * ((c + 1) % 3)], se = s6[1 + 2 * ((c + 1) % 3)];
                    Bh[m] = 1. / (invtau_R * mr + invtau_I * (mr * sh + mi));
                    Ah[m] = (invtau_R * mr - invtau_I * (mr * sh + mi)) * Bh[m];
                    Be[m] = 1. / (invtau_R * er + invtau_I * (er * se + ei));
                    Ae[m] = (invtau_R * er - invtau_I * (er * se + ei)) * Be[m];
                    const long a = c + 3L * address_notn[l] + 3 * n3;
                    if (Cont[l] == 'a') {
                        /* aux slot: the half driven along axis c+2 */
                        sh = s6[0 + 2 * ((c + 2) % 3)];
                        se = s6[1 + 2 * ((c + 2) % 3)];
                        Bh[a] = 1. / (invtau_R * mr + invtau_I * (mr * sh + mi));
                        Ah[a] = (invtau_R * mr - invtau_I * (mr * sh + mi)) * Bh[a];
                        Be[a] = 1. / (invtau_R * er + invtau_I * (er * se + ei));
                        Ae[a] = (invtau_R * er - invtau_I * (er * se + ei)) * Be[a];
                    }
                    if (Cont[l] == 'e' || Cont[l] == 'b') {
                        Be[a] = 1. / (0.5 * er - invtau_R * (0.5 * ei / invtau_I));
                        Ae[a] = -(0.5 * er + invtau_R * (0.5 * ei / invtau_I)) * Be[a];
                    }
                    if (Cont[l] == 'h' || Cont[l] == 'b') {
                        Bh[a] = 1. / (0.5 * mr - invtau_R * (0.5 * mi / invtau_I));
                        Ah[a] = -(0.5 * mr + invtau_R * (0.5 * mi / invtau_I)) * Bh[a];
                    }
                }
            }
}

/* ------------------------------------------------------------------------ */
/* time-step parameters: set_tau :515-524 */
void orc_set_tau(double omega, double min_Dt, int *N_2pi, double *invtau_R, double *invtau_I)
{
    int n = 0;
    while (omega * min_Dt * n <= ORC_TWO_PI) n++;
    const double dphi = ORC_TWO_PI / ((double)n);
    const double dt = dphi / omega;
    *N_2pi = n;
    *invtau_R = (0.5 * dphi) / (dt * sin(0.5 * dphi));
    *invtau_I = (0.5 * omega) / (cos(0.5 * dphi));
}

/* source envelope: set_env :452-475 (sin^2 ramp-up, flat, cos^2 ramp-down, zero) */
double orc_set_env(int N, const int tp[3], int jh, int jt, int jp)
{
    double f;
    const double t = 0.5 * ((double)jh) + ((double)jt);
    if (jp < tp[0]) {
        const double dphi = ORC_TWO_PI / ((double)4 * tp[0]);
        const double dphis = ORC_TWO_PI / ((double)4 * tp[0] * N);
        const double complex P = cexp(I * dphi * ((double)jp));
        const double complex Q = cexp(I * dphis * t);
        f = cimag(P * Q);
    } else if (jp < tp[0] + tp[1]) {
        f = 1.;
    } else if (jp < 2 * tp[0] + tp[1]) {
        const double dphi = ORC_TWO_PI / ((double)4 * tp[0]);
        const double dphis = ORC_TWO_PI / ((double)4 * tp[0] * N);
        const double complex P = cexp(I * dphi * ((double)jp - (tp[0] + tp[1])));
        const double complex Q = cexp(I * dphis * t);
        f = creal(P * Q);
    } else if (jp < tp[2]) {
        f = 0.;
    } else {
        return NAN;
    }
    const double norm = 1. / ((double)1 * (tp[0] + tp[1]) * N);
    return norm * f * f;
}

/* exp(i*phi) at whole and half steps: main :93-99 */
void orc_expn_table(int N, double complex *ExpN)
{
    const double dphi = ORC_TWO_PI / ((double)N);
    for (int j = 0; j < N; j++) {
        const double p0 = dphi * ((double)j);
        const double p5 = dphi * (0.5 + ((double)j));
        ExpN[0 + 2 * j] = cexp(I * p0);
        ExpN[1 + 2 * j] = cexp(I * p5);
    }
}

/* ------------------------------------------------------------------------ */
/* difference operators: ope_R :372-392, ope_Rd :393-413 and their aux-slot
 * variants ope_Rmap :330-350, ope_Rdmap :351-371. */
struct stencil {
    int off[3];   /* neighbour offset along each axis (wrapped) */
    double bp[3]; /* boundary factor iBc on the wrapped neighbour, else 1 */
};

/* dir = -1: backward neighbours (for H); dir = +1: forward neighbours (for E) */
static void make_stencil(const int L[4], const int iBc[3], const int j[3], int dir,
                         struct stencil *st)
{
    int stride = 1;
    for (int a = 0; a < 3; a++) {
        int jn;
        if (dir < 0) {
            jn = (j[a] - 1 + L[a]) % L[a];
            st->bp[a] = (j[a] == 0) ? (double)iBc[a] : 1.;
        } else {
            jn = (j[a] + 1) % L[a];
            st->bp[a] = (j[a] + 1 == L[a]) ? (double)iBc[a] : 1.;
        }
        st->off[a] = (jn - j[a]) * stride;
        stride *= L[a];
    }
}

/* slot of component 0 of cell l: 3*l in the main array, 3*map[l] in the aux */
static inline long slot(const int *map, long l) { return map ? 3L * map[l] : 3L * l; }

/* Half curls of F at cell l.  part 0: the term differentiated along axis c+1
 * ("+" half), part 1: along axis c+2 ("-" half), part 2: both.  dir < 0 gives
 * the backward form used for H, dir > 0 the forward form used for E. */
static void half_curl(int part, int dir, const struct stencil *st, long l,
                      const double *F, const int *map, double W[3])
{
    for (int c = 0; c < 3; c++) {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        const long here = slot(map, l);
        const long n1 = slot(map, l + st->off[a1]);
        const long n2 = slot(map, l + st->off[a2]);
        double w = 0.;
        if (dir < 0) {
            if (part != 1) w += +F[a2 + here] - st->bp[a1] * F[a2 + n1];
            if (part != 0) w += -F[a1 + here] + st->bp[a2] * F[a1 + n2];
        } else {
            if (part != 1) w += +st->bp[a1] * F[a2 + n1] - F[a2 + here];
            if (part != 0) w += -st->bp[a2] * F[a1 + n2] + F[a1 + here];
        }
        W[c] = w;
    }
}

int orc_main_calc(const int L[4], const double *Ah, const double *Bh,
                  const double *Ae, const double *Be, const int iBc[3],
                  double *H_t, double *E_t, const int iBTIin[4],
                  const double *Hi, const double *Ei, const double complex ExpN2[2],
                  double complex *HB, double complex *EB,
                  double complex *HT, double complex *ET,
                  const char *Cont, const int *address_notn)
{
    const int L0 = L[0], L1 = L[1], L2 = L[2];
    const long n3 = (long)L0 * L1 * L2;
    double *Haux = H_t + 3 * n3, *Eaux = E_t + 3 * n3;
    const double sgn = (double)(iBTIin[3] / abs(iBTIin[3]));
    double W[3];
    int j[3];

    /* H sweep :255-286 */
    for (j[2] = 0; j[2] < L2; j[2]++)
        for (j[1] = 0; j[1] < L1; j[1]++)
            for (j[0] = 0; j[0] < L0; j[0]++) {
                const long l = j[0] + (long)L0 * j[1] + (long)L0 * L1 * j[2];
                struct stencil st;
                make_stencil(L, iBc, j, -1, &st);
                const char k = Cont[l];
                if (k == 'n') {
                    half_curl(2, -1, &st, l, E_t, NULL, W);
                    if (j[2] == iBTIin[2]) {
                        const long p = 2 * (j[0] + (long)L0 * j[1]);
                        W[0] += sgn * Ei[1 + p];
                        W[1] -= sgn * Ei[0 + p];
                    }
                    for (int c = 0; c < 3; c++)
                        H_t[c + 3 * l] = Ah[c + 3 * l] * H_t[c + 3 * l] + Bh[c + 3 * l] * (-W[c]);
                    half_curl(2, -1, &st, l, Eaux, address_notn, W);
                    for (int c = 0; c < 3; c++) H_t[c + 3 * l] += Bh[c + 3 * l] * (-W[c]);
                } else if (k == 'a') {
                    for (int half = 0; half < 2; half++) {
                        const long s = half ? 3 * n3 + 3L * address_notn[l] : 3 * l;
                        half_curl(half, -1, &st, l, E_t, NULL, W);
                        for (int c = 0; c < 3; c++)
                            H_t[s + c] = Ah[s + c] * H_t[s + c] + Bh[s + c] * (-W[c]);
                        half_curl(half, -1, &st, l, Eaux, address_notn, W);
                        for (int c = 0; c < 3; c++) H_t[s + c] += Bh[s + c] * (-W[c]);
                    }
                } else if (k == 'h' || k == 'b') {
                    const long s = 3 * n3 + 3L * address_notn[l];
                    half_curl(2, -1, &st, l, E_t, NULL, W);
                    for (int c = 0; c < 3; c++) H_t[c + 3 * l] += 0.5 * H_t[c + s];
                    for (int c = 0; c < 3; c++)
                        H_t[c + s] = Ah[c + s] * H_t[c + s] + Bh[c + s] * (-W[c]);
                    for (int c = 0; c < 3; c++) H_t[c + 3 * l] += 0.5 * H_t[c + s];
                }
            }

    /* E sweep :287-317 */
    for (j[2] = 0; j[2] < L2; j[2]++)
        for (j[1] = 0; j[1] < L1; j[1]++)
            for (j[0] = 0; j[0] < L0; j[0]++) {
                const long l = j[0] + (long)L0 * j[1] + (long)L0 * L1 * j[2];
                struct stencil st;
                const char k = Cont[l];
                if (k == 'n') {
                    make_stencil(L, iBc, j, +1, &st);
                    half_curl(2, +1, &st, l, H_t, NULL, W);
                    if (j[2] == iBTIin[2]) {
                        const long p = 2 * (j[0] + (long)L0 * j[1]);
                        W[0] += sgn * Hi[1 + p];
                        W[1] -= sgn * Hi[0 + p];
                    }
                    for (int c = 0; c < 3; c++)
                        E_t[c + 3 * l] = Ae[c + 3 * l] * E_t[c + 3 * l] + Be[c + 3 * l] * W[c];
                    half_curl(2, +1, &st, l, Haux, address_notn, W);
                    for (int c = 0; c < 3; c++) E_t[c + 3 * l] += Be[c + 3 * l] * W[c];
                } else if (k == 'a') {
                    make_stencil(L, iBc, j, +1, &st);
                    for (int half = 0; half < 2; half++) {
                        const long s = half ? 3 * n3 + 3L * address_notn[l] : 3 * l;
                        half_curl(half, +1, &st, l, H_t, NULL, W);
                        for (int c = 0; c < 3; c++)
                            E_t[s + c] = Ae[s + c] * E_t[s + c] + Be[s + c] * W[c];
                        half_curl(half, +1, &st, l, Haux, address_notn, W);
                        for (int c = 0; c < 3; c++) E_t[s + c] += Be[s + c] * W[c];
                    }
                } else if (k == 'e' || k == 'b') {
                    /* the reference takes the BACKWARD difference of H here (:310) */
                    make_stencil(L, iBc, j, -1, &st);
                    const long s = 3 * n3 + 3L * address_notn[l];
                    half_curl(2, -1, &st, l, H_t, NULL, W);
                    for (int c = 0; c < 3; c++) E_t[c + 3 * l] += 0.5 * E_t[c + s];
                    for (int c = 0; c < 3; c++)
                        E_t[c + s] = Ae[c + s] * E_t[c + s] + Be[c + s] * W[c];
                    for (int c = 0; c < 3; c++) E_t[c + 3 * l] += 0.5 * E_t[c + s];
                }
            }

    /* running DFT on the two monitor planes :318-328.  A PML cell on a plane
     * makes the reference exit (:320); the oracle reports it and, like the
     * reference built with exit() made non-fatal, still accumulates. */
    const long pl = (long)L0 * L1;
    int rc = 0;
    for (long p = 0; p < pl; p++)
        if (Cont[p + pl * iBTIin[0]] == 'a' || Cont[p + pl * iBTIin[1]] == 'a') rc = -1;
    for (long p = 0; p < pl; p++)
        for (int v = 0; v < 2; v++) {
            HB[v + 2 * p] += ExpN2[0] * ((double complex)H_t[v + 3 * p + 3 * pl * iBTIin[0]]);
            EB[v + 2 * p] += ExpN2[1] * ((double complex)E_t[v + 3 * p + 3 * pl * iBTIin[0]]);
            HT[v + 2 * p] += ExpN2[0] * ((double complex)H_t[v + 3 * p + 3 * pl * iBTIin[1]]);
            ET[v + 2 * p] += ExpN2[1] * ((double complex)E_t[v + 3 * p + 3 * pl * iBTIin[1]]);
        }
    return rc;
}

/* ------------------------------------------------------------------------ */
/* the time loop of main :146-167 */
int orc_time_loop(const int L[4], const double *Ah, const double *Bh,
                  const double *Ae, const double *Be, const int iBc[3],
                  double *H_t, double *E_t, const int iBTIin[4],
                  const double complex *Hinc, const double complex *Einc,
                  int N, const int tp[3], int k_begin, int k_end,
                  double complex *HB, double complex *EB,
                  double complex *HT, double complex *ET,
                  const char *Cont, const int *address_notn)
{
    const long np = 2L * L[0] * L[1];
    double complex *ExpN = malloc(sizeof(double complex) * 2 * N);
    double *Hi = malloc(sizeof(double) * np);
    double *Ei = malloc(sizeof(double) * np);
    int rc = 0;
    if (!ExpN || !Hi || !Ei) { rc = -2; goto done; }
    orc_expn_table(N, ExpN);
    for (int k = k_begin; k < k_end; k++) {
        const int jp = k / N, jt = k % N;
        const int jn = (jt + 1) % N;
        for (long p = 0; p < np; p++) {
            Ei[p] = (2.) * orc_set_env(N, tp, 1, jt, jp) * creal(conj(ExpN[1 + 2 * jt]) * Einc[p]);
            Hi[p] = (2.) * orc_set_env(N, tp, 0, (jt + 1), jp) * creal(conj(ExpN[0 + 2 * jn]) * Hinc[p]);
        }
        if (orc_main_calc(L, Ah, Bh, Ae, Be, iBc, H_t, E_t, iBTIin, Hi, Ei, &ExpN[2 * jn],
                          HB, EB, HT, ET, Cont, address_notn))
            rc = -1;
    }
done:
    free(ExpN);
    free(Hi);
    free(Ei);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* mode overlap S = tilXi^H (HB_x, HB_y, -EB_y, EB_x): S_calc :437-445 */
void orc_overlap(const int L[4], int n_cols, const double complex *t,
                 const double complex *HB, const double complex *EB, double complex *S)
{
    const long pl = (long)L[0] * L[1];
    const long na = 2 * pl, ld = 2 * na;
    for (int col = 0; col < n_cols; col++) {
        double complex acc = 0.;
        const double complex *tc = t + ld * col;
        for (long r = 0; r < pl; r++) {
            acc += conj(tc[r]) * HB[0 + 2 * r];
            acc += conj(tc[r + pl]) * HB[1 + 2 * r];
            acc += conj(tc[r + na]) * (-EB[1 + 2 * r]);
            acc += conj(tc[r + pl + na]) * EB[0 + 2 * r];
        }
        S[col] = acc;
    }
}
