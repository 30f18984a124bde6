/*
 * CPU oracle for the split-field FDTD time loop -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C99 restatement of the reference algorithm in
 * FDTDcalc/FDTDsplitfieldMetal.c (SMatrAnEM).  It is the checker for the
 * CUDA path: only tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py may load it.  Nothing in the product links or calls it.
 *
 * Parity: pinned bit-for-bit against the reference compiled from its own
 * sources (oracle/Makefile -> oracle/_ref/) and against the golden vectors in
 * tests/golden/ that were generated from it.
 *
 * Array conventions follow the reference exactly:
 *   complex arrays are interleaved (re, im) doubles (C99 double complex);
 *   cell index l = j0 + L0*j1 + L0*L1*j2; component c of cell l at c + 3*l;
 *   the aux (split / stable-form) slot of cell l sits at 3*L3D + 3*address_notn[l]
 *   with L3D = L0*L1*L2; address_notn[l] == Lnotn marks an ordinary ('n') cell
 *   whose aux slot is the zero sentinel.
 */
#ifndef SMATRAN_FDTD_ORACLE_H
#define SMATRAN_FDTD_ORACLE_H

#include <complex.h>

#ifdef __cplusplus
extern "C" {
#endif

/* sigma[2*(L0+L1+L2)] from the stretched media (reference set_sigma :858-926). */
void orc_set_sigma(const int L[4], const double complex *mu, const double complex *epsi,
                   double *sigma);
/* divides the PML stretch out of mu, epsi in place (reference remove_sigma :822-853).
 * Returns 0, or -1 where the reference would exit ("mu/epsi error"). */
int orc_remove_sigma(const int L[4], double complex *mu, double complex *epsi,
                     const double *sigma);
/* cell classes 'n','a','h','e','b' and compact aux addresses; returns Lnotn
 * (reference set_address :188-233). */
int orc_set_address(const int L[4], const double *sigma, const double complex *mu,
                    const double complex *epsi, char *Cont, int *address_notn);
/* update coefficients, arrays of 3*(L3D+Lnotn) doubles zero-filled by the caller
 * (reference main :106-143). */
void orc_coefficients(const int L[4], int Lnotn, const double *sigma,
                      const double complex *mu, const double complex *epsi,
                      const char *Cont, const int *address_notn,
                      double invtau_R, double invtau_I,
                      double *Ah, double *Bh, double *Ae, double *Be);
/* time-step parameters (reference set_tau :515-524). */
void orc_set_tau(double omega, double min_Dt, int *N_2pi, double *invtau_R, double *invtau_I);
/* source envelope (reference set_env :452-475); returns NaN where the reference exits. */
double orc_set_env(int N_2pi, const int time_period[3], int j_half, int j_time, int j_period);
/* exp(i*phi) table of 2*N_2pi entries (reference main :93-99). */
void orc_expn_table(int N_2pi, double complex *ExpN);

/* One Yee step (reference main_calc :242-329).  Returns 0, or -1 where the
 * reference would exit because a monitor plane holds a PML ('a') cell. */
int orc_main_calc(const int L[4], const double *Ah, const double *Bh,
                  const double *Ae, const double *Be, const int iBc[3],
                  double *H_t, double *E_t, const int iBTIin[4],
                  const double *Hi, const double *Ei, const double complex ExpN2[2],
                  double complex *HB, double complex *EB,
                  double complex *HT, double complex *ET,
                  const char *Cont, const int *address_notn);

/* The reference time loop (main :146-167) over steps [k_begin, k_end) of the
 * global step counter k = j_period*N_2pi + j_time, with the incident profile
 * Hinc/Einc (complex, 2*L0*L1 each).  H_t/E_t hold 3*(L3D+Lnotn+1) doubles. */
int orc_time_loop(const int L[4], const double *Ah, const double *Bh,
                  const double *Ae, const double *Be, const int iBc[3],
                  double *H_t, double *E_t, const int iBTIin[4],
                  const double complex *Hinc, const double complex *Einc,
                  int N_2pi, const int time_period[3], int k_begin, int k_end,
                  double complex *HB, double complex *EB,
                  double complex *HT, double complex *ET,
                  const char *Cont, const int *address_notn);

/* Mode-overlap projection for one monitor plane given the first n_cols
 * columns of the tilde-Xi matrix, column-major with leading dimension 4*L0*L1
 * (reference S_calc :437-445). */
void orc_overlap(const int L[4], int n_cols, const double complex *tilXi_cols,
                 const double complex *HB, const double complex *EB, double complex *S);

#ifdef __cplusplus
}
#endif
#endif
