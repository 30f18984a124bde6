/*
 * LAPACK entry points for linking the reference mode solver (ModeCalc/Mcalc.c)
 * into oracle/_ref/Mcalc_ref.  TEST INFRASTRUCTURE ONLY.
 *
 * The image has no system LAPACK.  scipy's bundled OpenBLAS exports the
 * routines under a "scipy_" prefix with 32-bit integers; Mcalc declares
 * dgeev_/zgeev_ with `long` arguments (Mcalc.c:858-861, :937-940), so these
 * wrappers narrow the integers, pass the hidden Fortran string lengths and
 * widen INFO on the way back.  zgemm_ and dznrm2_ come from blas_shim.c.
 */
#include <complex.h>
#include <stddef.h>

extern void scipy_dgeev_(const char *jobvl, const char *jobvr, const int *n, double *a, const int *lda,
                         double *wr, double *wi, double *vl, const int *ldvl, double *vr, const int *ldvr,
                         double *work, const int *lwork, int *info, size_t, size_t);
extern void scipy_zgeev_(const char *jobvl, const char *jobvr, const int *n, double complex *a, const int *lda,
                         double complex *w, double complex *vl, const int *ldvl, double complex *vr,
                         const int *ldvr, double complex *work, const int *lwork, double *rwork, int *info,
                         size_t, size_t);

void dgeev_(char *jobvl, char *jobvr, long *n, double *a, long *lda, double *wr, double *wi, double *vl,
            long *ldvl, double *vr, long *ldvr, double *work, long *lwork, long *info)
{
    int n_ = (int)*n, lda_ = (int)*lda, ldvl_ = (int)*ldvl, ldvr_ = (int)*ldvr, lwork_ = (int)*lwork, info_ = 0;
    scipy_dgeev_(jobvl, jobvr, &n_, a, &lda_, wr, wi, vl, &ldvl_, vr, &ldvr_, work, &lwork_, &info_, 1, 1);
    *info = info_;
}

void zgeev_(char *jobvl, char *jobvr, long *n, double complex *a, long *lda, double complex *w,
            double complex *vl, long *ldvl, double complex *vr, long *ldvr, double complex *work, long *lwork,
            double *rwork, long *info)
{
    int n_ = (int)*n, lda_ = (int)*lda, ldvl_ = (int)*ldvl, ldvr_ = (int)*ldvr, lwork_ = (int)*lwork, info_ = 0;
    scipy_zgeev_(jobvl, jobvr, &n_, a, &lda_, w, vl, &ldvl_, vr, &ldvr_, work, &lwork_, rwork, &info_, 1, 1);
    *info = info_;
}

extern void scipy_zgesv_(const int *n, const int *nrhs, double complex *a, const int *lda, int *ipiv,
                         double complex *b, const int *ldb, int *info);

/* Smat/Scalc.c declares zgesv_ with int arguments (:315): a plain forward */
void zgesv_(int *n, int *nrhs, double complex *a, int *lda, int *ipiv, double complex *b, int *ldb, int *info)
{
    scipy_zgesv_(n, nrhs, a, lda, ipiv, b, ldb, info);
}
