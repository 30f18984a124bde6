/*
 * zgemm_ and dznrm2_ forwarded to scipy's bundled OpenBLAS, for linking the
 * reference S-matrix program (Smat/Scalc.c) into oracle/_ref/Scalc_ref, whose
 * layer transfer multiplies matrices of order 2*L0*L1 (the textbook loops of
 * blas_shim.c would take minutes there).  TEST INFRASTRUCTURE ONLY.
 */
#include <complex.h>
#include <stddef.h>

extern void scipy_zgemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k,
                         const double complex *alpha, const double complex *A, const int *lda,
                         const double complex *B, const int *ldb, const double complex *beta, double complex *C,
                         const int *ldc, size_t, size_t);
extern double scipy_dznrm2_(const int *n, const double complex *x, const int *incx);

void zgemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k, const double complex *alpha,
            const double complex *A, const int *lda, const double complex *B, const int *ldb,
            const double complex *beta, double complex *C, const int *ldc)
{
    scipy_zgemm_(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, 1, 1);
}

double dznrm2_(const int *n, const double complex *x, const int *incx) { return scipy_dznrm2_(n, x, incx); }
