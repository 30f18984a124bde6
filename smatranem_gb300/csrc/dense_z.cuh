/* Private to the library: dense complex FP64 kernels (dense_z.cu) used by the
 * layer-transfer S matrix (scalc.cu).  Column-major with leading dimensions;
 * every call is ordered on stream st. */
#ifndef SMATRAN_DENSE_Z_CUH
#define SMATRAN_DENSE_Z_CUH

#include <cuda_runtime.h>

namespace smat {
namespace dense {

/* How the multiply-adds run: tc = 1, FP64-accurate products on the tensor
 * cores (zgemm_tc.cu; ws / ws_bytes: workspace for products up to the sizes
 * tc_workspace_bytes was asked for; err: a device int the kernel's bounded
 * waits set on a timeout), tc = 0, the FP64 multiply-add kernel. */
struct GemmCtx {
    int tc;
    void *ws;
    size_t ws_bytes;
    int *err;
    unsigned wait_limit = 0; /* polls of a bounded wait (0: the default) */
    int skip_pair = -1;      /* >= 0: the timeout test leaves that slice pair unloaded */
};

/* C += alpha * A * B, A m x k, B k x n (g null: the FP64 kernel) */
int zgemm_acc(int m, int n, int k, double2 alpha, const double2 *A, int lda, const double2 *B, int ldb, double2 *C,
              int ldc, const GemmCtx *g, cudaStream_t st);
/* the tensor-core product itself, and its workspace for products up to m x n */
int zgemm_acc_tc(int m, int n, int k, double2 alpha, const double2 *A, int lda, const double2 *B, int ldb, double2 *C,
                 int ldc, const GemmCtx &g, cudaStream_t st);
size_t tc_workspace_bytes(int m, int n);
/* whether this device gives the tensor-core product its shared memory */
bool tc_available();
/* the process-wide choice of smat_scalc and smat_zgesv (smat_dense_mode) */
int dense_mode();
/* a context for products up to m x n in the process-wide mode (the FP64
 * kernel where the mode is 0 or the device lacks the tensor-core form's
 * shared memory); check after synchronising; release frees it */
int gemm_ctx_alloc(GemmCtx &g, int m, int n, cudaStream_t st);
int gemm_ctx_check(const GemmCtx &g);
void gemm_ctx_release(GemmCtx &g);
/* out (n x m) = in^T or in^H (in: m x n) */
int transpose(int m, int n, const double2 *in, int ldi, double2 *out, int ldo, bool conj, cudaStream_t st);
/* LU with partial pivoting in place (LAPACK zgetrf semantics: ipiv[k] = row
 * exchanged with k, 0-based; *info (device) = first zero pivot, 1-based, or 0) */
int getrf(int n, double2 *A, int lda, int *ipiv, int *info, const GemmCtx *g, cudaStream_t st);
/* B <- A^{-1} B from getrf's factors */
int getrs(int n, int nrhs, const double2 *LU, int lda, const int *ipiv, double2 *B, int ldb, const GemmCtx *g,
          cudaStream_t st);

} // namespace dense
} // namespace smat

#endif
