/* Private to the library: dense complex FP64 kernels (dense_z.cu) used by the
 * layer-transfer S matrix (scalc.cu).  Column-major with leading dimensions;
 * every call is ordered on stream st. */
#ifndef SMATRAN_DENSE_Z_CUH
#define SMATRAN_DENSE_Z_CUH

#include <cuda_runtime.h>

namespace smat {
namespace dense {

/* C += alpha * A * B, A m x k, B k x n */
int zgemm_acc(int m, int n, int k, double2 alpha, const double2 *A, int lda, const double2 *B, int ldb, double2 *C,
              int ldc, cudaStream_t st);
/* out (n x m) = in^T or in^H (in: m x n) */
int transpose(int m, int n, const double2 *in, int ldi, double2 *out, int ldo, bool conj, cudaStream_t st);
/* LU with partial pivoting in place (LAPACK zgetrf semantics: ipiv[k] = row
 * exchanged with k, 0-based; *info (device) = first zero pivot, 1-based, or 0) */
int getrf(int n, double2 *A, int lda, int *ipiv, int *info, cudaStream_t st);
/* B <- A^{-1} B from getrf's factors */
int getrs(int n, int nrhs, const double2 *LU, int lda, const int *ipiv, double2 *B, int ldb, cudaStream_t st);

} // namespace dense
} // namespace smat

#endif
