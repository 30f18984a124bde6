/*
 * Private to the library: the plan object (device-resident state of one
 * structure and its batch of excitations) and the helpers that launch its
 * steps.  Shared by the plan and adjoint translation units; not part of the
 * C ABI (include/smatran_fdtd.h sees only an opaque smat_fdtd_plan).
 */
#ifndef SMATRAN_PLAN_INTERNAL_CUH
#define SMATRAN_PLAN_INTERNAL_CUH

#include <cuda_runtime.h>

#include <vector>

#include "fdtd_internal.cuh"
#include "host_internal.h"
#include "smatran_fdtd.h"

namespace smat {
namespace plan {

constexpr int GRAPH_STEPS = 32; /* steps per captured graph (= FP32 ring length) */
constexpr int RING_K = 32;

inline int cuda_fail(cudaError_t e, const char *what)
{
    return smat_fail(SMAT_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call)                                                                                                       \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) return smat::plan::cuda_fail(e_, #call);                                              \
    } while (0)

/* zero-filled device allocation, ordered on stream st */
template <class T> inline int dalloc(T **p, size_t n, cudaStream_t st)
{
    *p = nullptr;
    if (n == 0) return SMAT_OK;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return smat_fail(SMAT_ENOMEM, "cudaMalloc of %zu bytes: %s", n * sizeof(T), cudaGetErrorString(e));
    }
    e = cudaMemsetAsync(*p, 0, n * sizeof(T), st);
    if (e != cudaSuccess) return smat_fail(SMAT_ECUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    return SMAT_OK;
}

} // namespace plan
} // namespace smat

struct smat_fdtd_plan {
    int L[4], iBc[3], iBTIin[4];
    int precision, batch, lnotn;
    long long n3;
    int pl;
    double invtau_R = 0, invtau_I = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    long long dev_bytes = 0;
    std::vector<char> cont;    /* host copy of the cell classes */
    std::vector<int> addr;     /* host copy of address_notn */

    /* common device state */
    int *d_base = nullptr;
    double *d_inc = nullptr;   /* [batch][8*pl] */
    double *d_xsrc = nullptr;  /* explicit sheet planes */
    double *d_xphase = nullptr;
    float *d_xphase32 = nullptr;
    double *d_sched = nullptr; /* [nsched][6] */
    int nsched = 0;
    double *d_phase = nullptr; /* [nsched][nfreq][4] */
    float *d_phase32 = nullptr;
    double *d_acc = nullptr;   /* [batch][nfreq][nq][4][pl] complex */
    float *d_ring = nullptr;
    int nfreq = 0, nq = 0, planes[smat::MAX_PLANES] = {0};
    bool ref_dft = false;      /* DFT slot 0 on planes (iB, iT) is the reference one */
    bool ref_planes_ok = false; /* no PML cell on iB, iT (else the reference exits, :320) */
    double *d_scratch = nullptr;
    int *d_iI = nullptr;      /* [batch] source plane per excitation */
    std::vector<int> h_iI;    /* host copy */
    double *d_isgn = nullptr; /* [batch] its sign */

    /* FP64 */
    uint8_t *d_flags = nullptr;
    int *d_addr = nullptr;
    double *d_cm = nullptr, *d_ca = nullptr;
    double *d_H64 = nullptr, *d_E64 = nullptr, *d_Ha64 = nullptr, *d_Ea64 = nullptr;

    /* FP32 */
    float *d_bh = nullptr, *d_be = nullptr, *d_tab = nullptr;
    uint8_t *d_pmask = nullptr;
    smat::Rec32 *d_hrec = nullptr, *d_erec = nullptr;
    float *d_H32 = nullptr, *d_E32 = nullptr, *d_Ha32 = nullptr, *d_Ea32 = nullptr;
    float *d_H32b = nullptr, *d_E32b = nullptr, *d_Ha32b = nullptr, *d_Ea32b = nullptr; /* second set */
    int cur = 0;          /* FP32: which field set holds the current state */
    int *d_qorder = nullptr; /* kernel 6: quads with a PML x index first (nqp of them), then the others */
    int nqp = 0;
    int nrec_metal = 0;   /* records of stable-form or frozen components (metal cells) */
    int *d_hmetal = nullptr, *d_emetal = nullptr; /* kernel 6: cells of those records, H and E side */
    int nhmetal = 0, nemetal = 0;
    int nrec_split = 0;   /* records of split cells (lossy media in a PML) */
    int nstable = 0;
    int *d_hgen = nullptr, *d_egen = nullptr; /* record (general) cells of each sweep, in cell order */
    int nhgen = 0, negen = 0;
    std::vector<int> hgen_z, egen_z; /* [L2+1]: index of the first general cell of plane z */
    int szc = 0; /* sweeps (kernels 0, 2): planes per H/E chunk, 0 = whole grid */
    int sweep_mb = 5; /* vectorised sweep register bound: minimum resident blocks 5, 6 or 8 */
    bool adj_scalar = false; /* FP32 adjoint: scalar kernels even where the vectorised ones apply */
    std::vector<int> hgen_host, egen_host; /* host copies of the general-cell lists */
    /* FP32 launch configuration (autotuned): two sweeps (0), two vectorised
     * sweeps (2, needs L0 % 4 == 0), the whole-row fused step (6); ns is the
     * fifth tuning value, unused by these forms */
    int fused = 0, ty = 8, zc = 40, ns = 4, ctas_per_sm = 0;
    int max_ctas = -1; /* cached occupancy of the current configuration */
    int *d_err = nullptr; /* device error flag */
    int by32 = 8;

    /* graphs: a chunk of GRAPH_STEPS steps, position independent via d_base */
    cudaGraphExec_t graph = nullptr;
    bool graph_failed = false;

    std::vector<void *> allocations;

    /* bytes copied between host and device on behalf of this plan (uploads
     * at creation, sources, schedules, read-backs), for smat_fdtd_copy_bytes */
    long long h2d_bytes = 0, d2h_bytes = 0;
    cudaError_t cpy(void *dst, const void *src, size_t n, cudaMemcpyKind kind)
    {
        if (kind == cudaMemcpyHostToDevice) h2d_bytes += (long long)n;
        else if (kind == cudaMemcpyDeviceToHost) d2h_bytes += (long long)n;
        return cudaMemcpyAsync(dst, src, n, kind, stream);
    }

    template <class T> int alloc(T **p, size_t n)
    {
        int rc = smat::plan::dalloc(p, n, stream);
        if (rc == SMAT_OK && *p) {
            allocations.push_back((void *)*p);
            dev_bytes += (long long)(n * sizeof(T));
        }
        return rc;
    }
};

namespace smat {
namespace plan {
Geo make_geo(const smat_fdtd_plan *p);
P64 make_p64(const smat_fdtd_plan *p, bool xp);
P32 make_p32(const smat_fdtd_plan *p, bool xp);
Row32 make_row(const smat_fdtd_plan *p, bool xp);
/* the launches of steps rel0 .. rel0+n-1 relative to *d_base (no bump) */
void enqueue_steps(smat_fdtd_plan *p, int rel0, int n, bool xp);
void sweep_step(smat_fdtd_plan *p, const P32 &q, int rel, cudaStream_t st);
void enqueue_update(smat_fdtd_plan *p, int rel, cudaStream_t st);
/* one step of form 6 on stream st: the fused launch, the metal-cell launch
 * after it (plans with metal cells), then the field sets swap */
void launch_row_step(smat_fdtd_plan *p, bool xp, int rel, cudaStream_t st);
int sm_count();
void drop_graph(smat_fdtd_plan *p);
} // namespace plan
} // namespace smat

#endif
