/*
 * Minimal BLAS entry points for linking the reference FDTD into oracle/_ref/.
 * TEST INFRASTRUCTURE ONLY.
 *
 * FDTDcalc/FDTDsplitfieldMetal.c calls zgemm_ and dznrm2_ only inside its
 * check_Xi diagnostic (:528-553), whose result is printed to stderr and never
 * feeds the time loop.  These are textbook triple loops (no blocking, no
 * threads) so that the reference builds with no external BLAS library.
 */
#include <complex.h>
#include <math.h>

static double complex op(char t, const double complex *A, int ld, int i, int j)
{
    /* element (i, j) of op(A) for column-major A */
    if (t == 'N' || t == 'n') return A[i + (long)ld * j];
    if (t == 'T' || t == 't') return A[j + (long)ld * i];
    return conj(A[j + (long)ld * i]);
}

void zgemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k,
            const double complex *alpha, const double complex *A, const int *lda,
            const double complex *B, const int *ldb, const double complex *beta,
            double complex *C, const int *ldc)
{
    for (int j = 0; j < *n; j++)
        for (int i = 0; i < *m; i++) {
            double complex acc = 0.;
            for (int p = 0; p < *k; p++) acc += op(*ta, A, *lda, i, p) * op(*tb, B, *ldb, p, j);
            double complex *c = &C[i + (long)(*ldc) * j];
            *c = (*beta == 0.) ? *alpha * acc : *alpha * acc + *beta * *c;
        }
}

double dznrm2_(const int *n, const double complex *x, const int *incx)
{
    double s = 0.;
    for (int i = 0; i < *n; i++) {
        const double complex v = x[(long)i * (*incx)];
        s += creal(v) * creal(v) + cimag(v) * cimag(v);
    }
    return sqrt(s);
}

/* exit() replacement for the shared-object build (see ref_prelude.h) */
int ref_exit_calls = 0;
int ref_last_exit_code = 0;
void ref_soft_exit(int code)
{
    ref_exit_calls++;
    ref_last_exit_code = code;
}
