/*
 * Internal device-side data layout of a plan (shared by the kernel and the
 * plan translation units).
 *
 * HBM layout, per excitation b of the batch (all structure-of-arrays, cell
 * index l = j0 + L0*j1 + L0*L1*j2, x fastest so a warp reads 32 consecutive
 * cells of one component):
 *
 *   FP64 (bit-identical path, the reference's representation):
 *     H, E   [3][L3D] doubles    main slot (total field of ordinary cells)
 *     Ha, Ea [3][Lnotn+1]        aux slot of each non-'n' cell, compact in
 *                                 address_notn order, then a zero sentinel
 *     coefficients: main [4][3][L3D] (Ah, Bh, Ae, Be), aux [4][3][Lnotn]
 *     flags  [L3D] bytes: cell class + "a neighbour has an aux slot" bits
 *
 *   FP32 (bandwidth path): total-field form.
 *     H, E   [3][L3D] floats     main + aux: what every neighbour's curl reads
 *     Ha, Ea [3][L3D] floats     aux slot (dense; written only by non-'n' cells)
 *     bh, be [3][L3D] floats     1/(tau_R^-1 * Re mu) (resp. epsi) per component:
 *                                 the only per-cell coefficient of ordinary cells
 *                                 (their A is exactly 1); split-PML cells scale it
 *                                 by 1-D sigma tables; cells needing anything else
 *                                 carry NaN in component 0 and a record index in
 *                                 component 1 ("general" cells, a short list)
 */
#ifndef SMATRAN_FDTD_INTERNAL_CUH
#define SMATRAN_FDTD_INTERNAL_CUH

#include <cstdint>
#include <cuda_runtime.h>

namespace smat {

enum : uint8_t { CLS_N = 0, CLS_A = 1, CLS_H = 2, CLS_E = 3, CLS_B = 4 };
constexpr uint8_t FL_BWD = 8;  /* a backward neighbour (wrapped) is non-'n' */
constexpr uint8_t FL_FWD = 16; /* a forward neighbour (wrapped) is non-'n' */

constexpr int MAX_PLANES = 8;

struct Geo {
    int L0, L1, L2, pl; /* pl = L0*L1 */
    long long n3;       /* L0*L1*L2 */
    int bc[3];          /* iBc */
    int iI;             /* source plane */
    double sgn;         /* iBTIin[3]/|iBTIin[3]| */
};

/* Per-step sources.  Step k of a launch = *base + rel. */
struct Src {
    const int *base;
    const double *sched; /* [nsched][6] {sE, cE, dE, sH, cH, dH} */
    const double *inc;   /* [batch][8*pl]: Hinc (2*pl complex) then Einc */
    const double *xsrc;  /* explicit planes {Hi[2*pl], Ei[2*pl]} or null */
    const int *iI;       /* [batch] source plane of each excitation (main :84 iI) */
    const double *sgn;   /* [batch] its sign, inci_mode/|inci_mode| (:253) */
};

struct Dft {
    int nfreq, nq;
    int planes[MAX_PLANES];
    const double *phase;  /* [nsched][nfreq][4] {pH re, im, pE re, im} */
    const float *phase32; /* FP32 flush: [nsched][nfreq][H, E]{hi re, hi im, lo re, lo im},
                           * hi = fl(phase), lo = fl(phase - hi) */
    const double *xphase; /* explicit {pH, pE} for smat_fdtd_step, or null */
    const float *xphase32; /* the same pairs of the explicit phases, [H, E][4] */
    double *acc;          /* [batch][nfreq][nq][4][pl] complex */
    int ringK;            /* FP32: samples kept per flush */
    float *ring;          /* FP32: [batch][ringK][nq][4][pl] */
};

struct P64 {
    Geo g;
    int batch, lnotn;
    const uint8_t *flags;
    const int *addr;
    const double *cm; /* [4][3][n3] */
    const double *ca; /* [4][3][lnotn] */
    double *H, *E;    /* [batch][3][n3] */
    double *Ha, *Ea;  /* [batch][3][lnotn+1] */
    Src s;
    Dft d;
};

/* A cell the FP32 fast path does not cover by its three per-cell numbers. */
struct Rec32 {
    float A0[3], B0[3]; /* main slot ("+" half of a split cell) */
    float A1[3], B1[3]; /* aux slot ("-" half, or the stable-form increment) */
    int kind;
    int pad[3];
};
enum : int { RK_N = 0, RK_A = 1, RK_STABLE = 2, RK_FROZEN = 3 };

struct P32 {
    Geo g;
    int batch;
    const float *bh, *be;
    const Rec32 *hrec, *erec;
    const float *tab;       /* [4][S]: A_h, G_h, A_e, G_e; S = L0+L1+L2 */
    const uint8_t *pmask;   /* [S]: axis index lies in a PML (either half) */
    float *H, *E, *Ha, *Ea; /* [batch][3][n3] */
    Src s;
    Dft d;
};

/* Several FP32 plans stepped together (a group): one vectorised-sweep launch
 * covers the cells of every member; block ranges and general-cell ranges per
 * member are prefix sums.  Loaded into a constant-memory table before the
 * group's launches (load_group32). */
constexpr int MAX_GROUP = 32;
struct Group32 {
    int n, by;
    int blk[MAX_GROUP + 1];                  /* first block of member m */
    int gen_h[MAX_GROUP + 1], gen_e[MAX_GROUP + 1]; /* first general (cell, excitation) of member m */
    const int *hgen[MAX_GROUP], *egen[MAX_GROUP];
    int nhgen[MAX_GROUP], negen[MAX_GROUP];
    P32 p[MAX_GROUP];
};

/* The work of one CTA of launch form 6 (excitation aside): pieces (row tile yt,
 * planes [z0, z1)).  With z chunks (zc > 0) one piece, item gidx = row tile
 * fastest, then z chunk.  Persistent (zc == 0): ngroups groups of one CTA per
 * excitation; group gidx takes row tile round * ngroups + gidx, whole, in each
 * full round (adjacent tiles run together, so their halo rows are read from
 * L2), then an equal share of the planes of the tiles left over.  Shared by the
 * kernel and the host's check of the partition (smat_row32_pieces). */
struct RowPieces {
    int G, R; /* groups, full rounds */
    long long u, uhi;
    int round;
    bool first;
    __host__ __device__ RowPieces(int nyt, int L2, int zc, int ngroups, int gidx)
        : G(ngroups > 0 ? ngroups : 1), R(zc > 0 ? 0 : nyt / (ngroups > 0 ? ngroups : 1)), round(0), first(true)
    {
        const long long lrem = (long long)(nyt - R * G) * L2;
        u = (long long)gidx * lrem / G;
        uhi = (long long)(gidx + 1) * lrem / G;
    }
    /* the next piece, or false; nyt, L2, zc and gidx as given to the constructor */
    __host__ __device__ bool next(int nyt, int L2, int zc, int gidx, int &yt, int &z0, int &z1)
    {
        if (zc > 0) {
            if (!first) return false;
            yt = gidx % nyt;
            z0 = gidx / nyt * zc;
            z1 = z0 + zc < L2 ? z0 + zc : L2;
        } else if (round < R) {
            yt = round * G + gidx;
            z0 = 0;
            z1 = L2;
            round++;
        } else if (u < uhi) {
            yt = R * G + (int)(u / L2);
            z0 = (int)(u % L2);
            z1 = (int)(L2 < z0 + (uhi - u) ? L2 : z0 + (uhi - u));
            u += z1 - z0;
        } else {
            return false;
        }
        first = false;
        return true;
    }
};

/* launch form 6: the fused step over whole x rows (fdtd_row32.cu); reads the
 * field set in p, writes the other set */
struct Row32 {
    P32 p;
    float *Hn, *En, *Han, *Ean; /* new set */
    int ty, zc;                 /* rows per tile, planes per z chunk (0: persistent groups) */
    int nyt, nzc, nitems;       /* row tiles, z chunks, CTAs */
    int ngroups;                /* persistent: groups of one CTA per excitation */
    const int *qorder;          /* [L0/4]: quads whose x index lies in a PML, then the others */
    int nqp;                    /* how many of the first kind */
    int has_rec;                /* the plan has record cells (lossy, PEC or metal cells) */
    int worder;                 /* 1: the last two warps trade places with the two before them */
};

/* Several plans in one persistent launch of form 6 (a group's form 3): CTAs
 * first[m] .. first[m+1]-1 belong to member m, in groups of one CTA per
 * excitation that march the member's own persistent schedule (RowPieces with
 * r[m].ngroups groups, r[m].ty rows per tile).  Passed whole as a kernel
 * parameter (under 12 KB). */
struct RowGroup32 {
    int n;
    int first[MAX_GROUP + 1];
    Row32 r[MAX_GROUP];
};


/* The curl stencil of a cell: offsets of its forward (fwd) or backward
 * neighbour along each axis, wrapped at the grid's faces, and the boundary
 * factor iBc at a wrapped neighbour (else 1). */
struct Stn32 {
    long long o[3];
    float f[3];
};

__device__ __forceinline__ Stn32 make_stn32(const Geo &g, int j0, int j1, int j2, bool fwd)
{
    Stn32 st;
    const int j[3] = {j0, j1, j2};
    const int L[3] = {g.L0, g.L1, g.L2};
    long long stride = 1;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const bool edge = fwd ? (j[a] + 1 == L[a]) : (j[a] == 0);
        const int jn = fwd ? (edge ? 0 : j[a] + 1) : (edge ? L[a] - 1 : j[a] - 1);
        st.o[a] = (long long)(jn - j[a]) * stride;
        st.f[a] = edge ? (float)g.bc[a] : 1.0f;
        stride *= L[a];
    }
    return st;
}

/* Half curls of a field given by an accessor get(c, offset). */
template <bool FWD, class Get>
__device__ __forceinline__ void curl32(const Get &get, const Stn32 &st, float pl[3], float mi[3])
{
    const float here[3] = {get(0, 0), get(1, 0), get(2, 0)};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int a1 = (c + 1) % 3, a2 = (c + 2) % 3;
        const float n2 = st.f[a1] * get(a2, st.o[a1]);
        const float n1 = st.f[a2] * get(a1, st.o[a2]);
        if (!FWD) {
            pl[c] = here[a2] - n2;
            mi[c] = n1 - here[a1];
        } else {
            pl[c] = n2 - here[a2];
            mi[c] = here[a1] - n1;
        }
    }
}

/* launchers (one translation unit per precision) */
void launch_h64(const P64 &p, int rel, cudaStream_t st);
void launch_e64(const P64 &p, int rel, cudaStream_t st);
void launch_dft64(const P64 &p, int rel, cudaStream_t st);
void launch_h32(const P32 &p, int rel, int by, int z0, int z1, cudaStream_t st);
void launch_e32(const P32 &p, int rel, int by, int z0, int z1, cudaStream_t st);
void launch_flush32(const P32 &p, int rel_end, int count, cudaStream_t st);
/* mb: register bound of the vectorised sweep (minimum resident blocks: 5, 6 or 8) */
void launch_h32v(const P32 &p, int rel, int by, int mb, int z0, int z1, const int *gcells, int ngh, cudaStream_t st);
void launch_e32v(const P32 &p, int rel, int by, int mb, int z0, int z1, const int *gcells, int nge, cudaStream_t st);
void load_group32(const Group32 *host_pinned, cudaStream_t st);
void launch_group32v(const Group32 &gr, int rel, cudaStream_t st);
/* form 6: threads of a CTA (one per quad of its ty + 1 rows, rounded up to
 * whole warps), shared memory, resident CTAs of ty rows and z chunks of zc
 * planes at register bound mb (1, 2 or 3 CTAs per SM; 1 for plans with record
 * cells) */
int row32_threads(int L0, int ty);
size_t row32_smem(int L0, int ty, int zc);
int row32_max_ctas_per_sm(int L0, int ty, int mb, int zc, bool rec);
void launch_row32(const Row32 &r, int rel, int mb, cudaStream_t st);
/* the metal cells of a form-6 step, after it: nh H cells, ne E cells (lists
 * of cell indices with stable-form or frozen records) */
void launch_row_metal(const Row32 &r, int rel, const int *hcells, int nh, const int *ecells, int ne, cudaStream_t st);
/* the grouped launch, CTAs of `threads` = 384 (one per SM) or 192 (two per
 * SM): its resident CTAs per SM at smem bytes of shared memory (0: does not
 * fit), and the launch itself */
int row32_group_max_ctas_per_sm(int threads, size_t smem, bool rec);
void launch_row32_group(const RowGroup32 &g, int rel, int threads, int grid, size_t smem, bool rec, cudaStream_t st);
void launch_bump(int *base, int by, cudaStream_t st);
void launch_set(int *base, int value, cudaStream_t st);
void launch_maxabs(const void *x, long long n, int is_double, double *out, cudaStream_t st);

} // namespace smat

#endif
