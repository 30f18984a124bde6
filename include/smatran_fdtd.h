/*
 * smatran_fdtd.h -- C ABI of the GB300 (sm_103a) split-field FDTD time loop.
 *
 * Drop-in replacement for the hot path of SMatrAnEM's FDTD solver,
 * FDTDcalc/FDTDsplitfieldMetal.c.  The reference has no library interface:
 * its time loop (main :146-167) calls main_calc (:242-329) once per step with
 * host arrays.  This header exposes that seam:
 *
 *   smat_main_calc            one step with exactly main_calc's arguments (host
 *                             buffers, stateless, slow: for binding-level parity)
 *   smat_fdtd_create / ...    a plan that keeps the structure and the fields
 *                             resident in HBM and runs many steps per call
 *
 * Conventions (all from the reference):
 *   L[4] = {L0, L1, L2, L3}: cells along x, y, z and the number of outer
 *       (port) layers at each z end (main :57).
 *   cell index l = j0 + L0*j1 + L0*L1*j2; a 3-vector field component c of cell
 *       l sits at c + 3*l ("reference layout"); complex arrays are interleaved
 *       (re, im) doubles, i.e. C99 double complex.
 *   H_t, E_t: 3*(L3D + Lnotn + 1) doubles, L3D = L0*L1*L2: the main field, then
 *       the aux (split-PML "-" half or stable-form increment) slot of each
 *       non-'n' cell at 3*L3D + 3*address_notn[l], then a zero sentinel.
 *   Planes: HB/EB/HT/ET are 2*L0*L1 complex: component v (0 = x, 1 = y) of
 *       pixel p = j0 + L0*j1 at v + 2*p (main_calc :318-328).
 *
 * Every function returns 0 on success or a negative SMAT_E* code; nothing
 * calls exit().  smat_last_error() gives a message for the calling thread.
 * Device memory, streams and kernels are owned by the library; the caller
 * owns every host buffer.  One plan lives on one CUDA device and one stream.
 */
#ifndef SMATRAN_FDTD_H
#define SMATRAN_FDTD_H

#ifdef __cplusplus
extern "C" {
#endif

#define SMAT_OK 0
#define SMAT_EINVAL (-1)    /* bad argument or inconsistent sizes */
#define SMAT_ECUDA (-2)     /* CUDA runtime error (message has the detail) */
#define SMAT_ENOMEM (-3)    /* device or host allocation failed */
#define SMAT_EMONITOR (-4)  /* a monitor plane holds a PML ('a') cell: the
                               reference aborts with "iBTIin[m] error!" (:320) */
#define SMAT_ESTATE (-5)    /* call not valid for this plan (precision, no schedule...) */
#define SMAT_ENUMERIC (-6)  /* non-finite value detected in the fields */

#define SMAT_FP64 0 /* fields and coefficients in FP64, same operation order as the
                       reference: bit-identical results */
#define SMAT_FP32 1 /* fields in FP32 (packed coefficient stream); DFT accumulated
                       in FP64; results within a stated tolerance of FP64 */

/* Structure of one simulation, at the level of the reference's precompute
 * (main :62-143).  mu/epsi are the media AFTER remove_sigma (:76), i.e. real
 * (or lossy) values times the metric factors; sigma is the per-axis stretch
 * profile recovered by set_sigma (:75), 2*(L0+L1+L2) doubles laid out as
 * sigma[h + 2*j0], sigma[2*L0 + h + 2*j1], sigma[2*(L0+L1) + h + 2*j2] with
 * h = 0 for the H sub-point and h = 1 for the E sub-point. */
typedef struct smat_fdtd_desc {
    int L[4];
    int iBc[3];          /* BoundaryCondition B0..B2 in {-1, 0, 1} (input.txt) */
    int iBTIin[4];       /* {iB, iT, iI, inci_mode}: monitor planes, source plane,
                            signed mode number (main :84) */
    double invtau_R;     /* from set_tau (:515-524) */
    double invtau_I;
    const double *mu;    /* 3*L3D complex */
    const double *epsi;  /* 3*L3D complex */
    const double *sigma; /* 2*(L0+L1+L2) */
    const unsigned char *pec; /* optional, L3D bytes: nonzero forces Ae = Be = 0 on
                                 the E components of that (ordinary) cell */
    int precision;       /* SMAT_FP64 or SMAT_FP32 */
    int batch;           /* independent excitations sharing the structure, >= 1 */
} smat_fdtd_desc;

typedef struct smat_fdtd_plan smat_fdtd_plan;

/* Message describing the last error on the calling thread ("" if none). */
const char *smat_last_error(void);

/* Host precompute, restating main :62-143.  Callable without a GPU. ------- */

/* set_sigma :858-926: sigma (2*(L0+L1+L2), zeroed by the callee) from the
 * stretched media. */
int smat_set_sigma(const int L[4], const double *mu, const double *epsi, double *sigma);
/* remove_sigma :822-853, in place.  SMAT_EINVAL where the reference exits. */
int smat_remove_sigma(const int L[4], double *mu, double *epsi, const double *sigma);
/* set_address :188-233: Cont[L3D] in {'n','a','h','e','b'}, address_notn[L3D];
 * *Lnotn receives the number of non-'n' cells. */
int smat_set_address(const int L[4], const double *sigma, const double *mu,
                     const double *epsi, char *Cont, int *Lnotn, int *address_notn);
/* coefficient build of main :106-143 into Ah, Bh, Ae, Be of 3*(L3D+Lnotn)
 * doubles each (zeroed by the callee). */
int smat_coefficients(const int L[4], int Lnotn, const double *sigma, const double *mu,
                      const double *epsi, const char *Cont, const int *address_notn,
                      double invtau_R, double invtau_I,
                      double *Ah, double *Bh, double *Ae, double *Be);
/* set_tau :515-524. */
int smat_set_tau(double omega, double min_Dt, int *N_2pi, double *invtau_R, double *invtau_I);
/* omega = 2*pi/(wavelength*k0) exactly as input_Lf evaluates it (:740). */
double smat_omega(double wavelength, double k0);
/* set_env :452-475; returns NaN where the reference exits ("f_env error!"). */
double smat_set_env(int N_2pi, const int time_period[3], int j_half, int j_time, int j_period);

/* The reference seam. ----------------------------------------------------- */

/* One Yee step: same arguments, layouts and results as main_calc
 * (FDTDsplitfieldMetal.c:242-329), ExpN2 being 2 complex.  All pointers are
 * host memory; fields and DFT planes are updated in place.  Runs the FP64
 * kernels on the current device; uploads and downloads everything per call. */
int smat_main_calc(const int L[4], const double *Ah, const double *Bh,
                   const double *Ae, const double *Be, const int iBc[3],
                   double *H_t, double *E_t, const int iBTIin[4],
                   const double *Hi, const double *Ei, const double *ExpN2,
                   double *HB, double *EB, double *HT, double *ET,
                   const char *Cont, const int *address_notn);

/* Plans. ------------------------------------------------------------------ */

/* Build a plan from the media (runs set_address and the coefficient build on
 * the host, then uploads).  stream: a cudaStream_t, or NULL for a stream the
 * plan creates and owns. */
int smat_fdtd_create(const smat_fdtd_desc *desc, void *stream, smat_fdtd_plan **plan);

/* Build an FP64 plan straight from main_calc's coefficient arrays
 * (main :101-143 outputs), for callers that already ran the precompute. */
int smat_fdtd_create_from_coeffs(const int L[4], const double *Ah, const double *Bh,
                                 const double *Ae, const double *Be, const int iBc[3],
                                 const char *Cont, const int *address_notn, int Lnotn,
                                 const int iBTIin[4], int batch, void *stream,
                                 smat_fdtd_plan **plan);

int smat_fdtd_destroy(smat_fdtd_plan *plan);

/* Geometry of a plan: L (4), Lnotn, precision, batch.  Any pointer may be NULL. */
int smat_fdtd_info(const smat_fdtd_plan *plan, int L[4], int *Lnotn, int *precision,
                   int *batch);

/* Fields of excitation b in the reference layout (3*(L3D+Lnotn+1) doubles
 * each).  FP32 plans convert on the way. */
int smat_fdtd_set_fields(smat_fdtd_plan *plan, int b, const double *H_t, const double *E_t);
int smat_fdtd_get_fields(smat_fdtd_plan *plan, int b, double *H_t, double *E_t);

/* Checkpoint and resume.  No counterpart in the reference (its FDTD state is
 * never written).  save_state writes the plan's state -- the fields and aux
 * slots of every excitation and the running-DFT accumulators -- to a binary
 * file, exactly as held on the device; load_state restores it into a plan of
 * the same grid, precision, batch, split-cell count and DFT setup (refused
 * with SMAT_EINVAL otherwise), after which run(k, ...) continues from step k
 * with the bits an uninterrupted run would give (FP32: with the same launch
 * form; another form gives the same fields and DFT sums grouped differently,
 * equal to rounding).  Call them between runs (an FP32 run leaves no DFT
 * samples pending). */
int smat_fdtd_save_state(smat_fdtd_plan *plan, const char *path);
int smat_fdtd_load_state(smat_fdtd_plan *plan, const char *path);

/* One step with explicit sheet sources (main_calc's Hi, Ei: 2*L0*L1 doubles,
 * shared by every excitation) and DFT phases ExpN2 (2 complex).  Accumulates
 * the reference DFT (frequency slot 0 on planes iB, iT). */
int smat_fdtd_step(smat_fdtd_plan *plan, const double *Hi, const double *Ei,
                   const double *ExpN2);

/* Incident profile of excitation b: Hinc, Einc complex 2*L0*L1 each, the
 * arrays set_incident (:479-511) builds. */
int smat_fdtd_set_incident(smat_fdtd_plan *plan, int b, const double *Hinc,
                           const double *Einc);

/* Source plane and direction of excitation b (default: iBTIin[2] and the sign
 * of iBTIin[3] for every excitation).  Lets one batch hold the excitations of
 * several ports; the reference runs one (iI, inci_mode) per process. */
int smat_fdtd_set_source_plane(smat_fdtd_plan *plan, int b, int iI, int inci_mode);

/* The reference CW schedule: envelope set_env (:452-475) and phases ExpN
 * (:93-99) for stop-period*N_2pi steps, with the reference DFT (one
 * frequency, planes iB and iT, phases ExpN[(k+1)%N_2pi]) as frequency slot 0.
 * Replaces any earlier schedule and DFT setup and zeroes the accumulators.
 * SMAT_EMONITOR when iB or iT holds a PML cell (the reference exits, :320). */
int smat_fdtd_set_cw_schedule(smat_fdtd_plan *plan, int N_2pi, const int time_period[3]);

/* The reference CW run as a general schedule (what smat_fdtd_set_cw_schedule
 * installs): src 6*stop-period*N_2pi doubles, phase 4*stop-period*N_2pi. */
int smat_cw_schedule(int N_2pi, const int time_period[3], double *src, double *phase);

/* A general schedule of nsteps steps.  src: 6 doubles per step
 * {sE, cE, dE, sH, cH, dH}; the sheet sources of step k are
 *   Ei = sE*(cE*Re(Einc) + dE*Im(Einc)),  Hi = sH*(cH*Re(Hinc) + dH*Im(Hinc)),
 * the reference's 2*env*Re(conj(ExpN)*inc) with (cE, dE) = ExpN.
 * DFT: nfreq frequencies on nplanes z-planes (planes[], at most 8), phases 4
 * doubles per (step, frequency): the complex weight of H then of E at step k,
 * laid out [k][f][4].  nfreq may be 0.  Zeroes the accumulators.  Unlike the
 * reference DFT, a plane may cut the PML: split cells contribute their total
 * field (main + aux), other cells their main slot as in main_calc :322-325. */
int smat_fdtd_set_schedule(smat_fdtd_plan *plan, int nsteps, const double *src,
                           int nfreq, int nplanes, const int *planes, const double *phase);

/* Advance every excitation over global steps [k_begin, k_end) of the schedule.
 * Asynchronous on the plan's stream; CUDA-graph captured in chunks. */
int smat_fdtd_run(smat_fdtd_plan *plan, int k_begin, int k_end);

/* Block until the plan's stream is idle; reports asynchronous errors. */
int smat_fdtd_sync(smat_fdtd_plan *plan);

/* Reference DFT planes of excitation b (frequency slot 0, planes iB/iT), in
 * main_calc's layout.  Any pointer may be NULL. */
int smat_fdtd_get_monitor(smat_fdtd_plan *plan, int b, double *HB, double *EB,
                          double *HT, double *ET);

/* DFT accumulator of excitation b, frequency f, schedule plane index q:
 * out = 4*L0*L1 complex, components (Hx, Hy, Ex, Ey) each over L0*L1 pixels. */
int smat_fdtd_get_dft(smat_fdtd_plan *plan, int b, int f, int q, double *out);

/* Number of DFT frequencies and monitor planes of the current schedule. */
int smat_fdtd_dft_count(const smat_fdtd_plan *plan, int *nfreq, int *nplanes);

/* Device address of the DFT accumulator of excitation b, frequency f, plane q
 * (4*L0*L1 complex: Hx, Hy, Ex, Ey) and the distance in complex elements
 * between consecutive frequencies.  Valid until the next set_schedule. */
int smat_fdtd_dft_device(smat_fdtd_plan *plan, int b, int f, int q, const double **ptr,
                         long long *fstride);

/* Mode-overlap projection on the GPU, the S-parameter extraction of S_calc
 * (FDTDsplitfieldMetal.c:419-448): for nvec DFT planes (plane v at
 * dft + v*vec_stride complex elements, components Hx, Hy, Ex, Ey over npix
 * pixels) and ncols columns of tilde-Xi (column-major, 4*npix complex rows in
 * the reference's row order), S[v*ncols + c] = sum_r conj(tilXi[r, c]) *
 * (HB_x, HB_y, -EB_y, EB_x)[r].  All pointers are device memory; FP64; the
 * result is the same bits on every call.  Block partial sums go to scratch
 * memory the call allocates stream-ordered on `stream` (NULL: the legacy
 * default stream) and frees again. */
int smat_overlap(int npix, int ncols, int nvec, long long vec_stride, const double *tilXi,
                 const double *dft, double *S, void *stream);

/* No counterpart in the reference.  smat_overlap without any device
 * allocation, for callers that must not allocate at this point: a host
 * process whose device memory pool belongs to a framework that forbids other
 * code to call cudaMalloc, or a long-running loop that must not fail on
 * memory after start-up.  The block partial sums go to a static device array of
 * SMAT_OVERLAP_NOALLOC_MAX complex doubles (1 MiB, held on every device that
 * loads the library until exit); a call needing more (ncols * nvec * blocks,
 * blocks <= 64 and about 4*npix/1024) fails with SMAT_EINVAL before launching.
 * The first call on a device looks up the array's device address (no
 * allocation), and so does the first call after the device's context was
 * re-created (cudaDeviceReset); make such a call outside any stream capture.  All calls on
 * a device share the array: calls that overlap on the GPU (different streams,
 * no ordering) race and corrupt each other's results; calls ordered on one
 * stream are safe.  Results equal smat_overlap's bit for bit. */
#define SMAT_OVERLAP_NOALLOC_MAX 65536
int smat_overlap_noalloc(int npix, int ncols, int nvec, long long vec_stride, const double *tilXi,
                         const double *dft, double *S, void *stream);

/* The same for every frequency of plane q of excitation b of a plan, with
 * tilde-Xi columns and the result (nfreq*ncols complex) in host memory. */
int smat_fdtd_overlap(smat_fdtd_plan *plan, int b, int q, int ncols, const double *tilXi_host,
                      double *S_host);

/* Groups of structures. -----------------------------------------------------
 * No counterpart in the reference (it runs one structure per process, main
 * :32-187).  A group advances several FP32 plans -- structures of any size,
 * each with its own batch of excitations, schedule and DFT -- together, one
 * CUDA graph launch per 32 steps (see set_tuning for the launch forms inside
 * it, plus the general cells and each member's DFT flush).  Members need
 * L0 % 4 == 0 and stay usable on their own; results are bit-identical to
 * stepping each member alone.  At most 32 members;
 * the group launches on the first member's stream and waits for the others'
 * streams before each run. */
typedef struct smat_fdtd_group smat_fdtd_group;
int smat_fdtd_group_create(smat_fdtd_plan *const *plans, int nplans, smat_fdtd_group **group);
int smat_fdtd_group_destroy(smat_fdtd_group *group);
/* mode 0: one grouped sweep launch for all members (blocks find their member
 * by prefix sums); mode 1: every member's own sweep launches back to back on
 * the group's stream; mode 2: every member's own launch form (its
 * smat_fdtd_set_tuning: the whole-row fused step or the sweeps) on the
 * member's own stream, forked from the group's stream and joined back, so the
 * members run side by side; mode 3: one persistent launch of the whole-row
 * fused step per step for every member (at most one excitation per
 * resident CTA in all; members with metal cells add their second launch): the
 * resident CTAs are shared out in groups of one CTA per excitation, each
 * member's groups marching its own persistent schedule.  All are captured as
 * one graph per 32 steps.  block_y: rows per sweep block, 1..4 (modes 0, 1);
 * mode 3: CTAs of 384 threads, one per SM (1), or of 192, two per SM (2),
 * each member's tile the most whole rows that fit. */
int smat_fdtd_group_set_tuning(smat_fdtd_group *group, int mode, int block_y);
/* fastest {mode, block_y} over nsteps steps, after autotuning every member
 * (smat_fdtd_autotune: their launch form for mode 2); members must be at the
 * zero state and are left there */
int smat_fdtd_group_autotune(smat_fdtd_group *group, int nsteps, int best[2], double *best_ms);
/* steps [k_begin, k_end) of every member's schedule */
int smat_fdtd_group_run(smat_fdtd_group *group, int k_begin, int k_end);
int smat_fdtd_group_sync(smat_fdtd_group *group);

/* Adjoint gradient. ----------------------------------------------------------
 * No counterpart in the reference (it has no gradient).  The objective is
 *   J = sum_b |S_b|^2,  S_b = sum_r conj(t_b,r) x_b,r,  x = (HB_x, HB_y, -EB_y, EB_x)
 * of excitation b's DFT at frequency f on DFT plane slot q (the S_calc
 * projection, S_calc :437-445) with mode columns tilXi_cols: ncols = 1 column
 * for every excitation, or ncols = batch, column b for excitation b (4*L0*L1
 * complex each, rows in that order; a weight w_b enters as sqrt(w_b) t_b).  The call runs the plan's schedule from rest
 * (fields and DFT zeroed) for nsteps steps with a checkpoint every K steps,
 * then runs the discrete adjoint backwards, recomputing each K-step segment
 * from its checkpoint.  Returns J and, for each cell i of the box
 * [box[0],box[1]) x [box[2],box[3]) x [box[4],box[5]) (x fastest),
 *   grad[i]      = dJ/ds_i, where s_i scales the cell's permittivity,
 *                  epsi -> epsi * (1 + s_i) on all three components
 *                  (so dJ/d eps_r = grad / eps_r for epsi = eps_r * metric),
 *   grad_c[c][i] = the same per E component (optional, may be NULL).
 * Design cells must be ordinary ('n') cells and the plan must hold no
 * stable-form (metal) cells.  Afterwards the DFT holds the forward result and
 * the fields are those of the first checkpoint segment.  Device memory: one
 * state copy per checkpoint (ceil(nsteps/K) copies) plus four field arrays. */
int smat_fdtd_adjoint_grad(smat_fdtd_plan *plan, int nsteps, int K, int f, int q, int ncols,
                           const double *tilXi_cols, const int box[6], double *grad, double *grad_c, double *J);

/* The FDTD input deck and the drop-in program. ------------------------------
 * A deck is what the reference FDTD reads (main :44-99): input.txt (keys
 * Prefix, BoundaryCondition, ModeP, FDTD; input_file0 :759-781, plus the
 * optional "FDTD_GPU: precision = FP32" line the reference ignores), the
 * per-layer Med files (input_data :665-699), the Mode files (get_RealNum
 * :632-661) and the Xi files (set_Xi/set_tilXi :557-628).  Only the tilde-Xi
 * columns S_calc reports and the incident column are kept. */
typedef struct smat_deck smat_deck;
int smat_deck_load(const char *input_txt, smat_deck **deck);
void smat_deck_free(smat_deck *deck);
/* 1 if the deck came from its binary cache.  No counterpart in the reference:
 * with the extra input.txt line "FDTD_GPU: cache = y" the parsed arrays are
 * kept in <prefix>.smatdeck, keyed by every data file's size and modification
 * time and by the input.txt keys that select Xi columns, and reused by later
 * loads while that key matches. */
int smat_deck_from_cache(const smat_deck *deck);
/* L, {iB, iT, iI, inci_mode}, iBc, time_period, omega (2*pi/(lambda*k0)),
 * min_Dt (sqrt of the smallest "min Dt^2" header), Dt_factor, N_real of the
 * bottom and top mode files; any pointer may be NULL. */
int smat_deck_info(const smat_deck *deck, int L[4], int iBTIin[4], int iBc[3], int time_period[3],
                   double *omega, double *min_dt, double *dt_factor, int nreal[2]);
/* mu, epsi (3*L3D complex, as stored: stretched), Hinc, Einc (2*L0*L1 complex). */
int smat_deck_arrays(const smat_deck *deck, double *mu, double *epsi, double *Hinc, double *Einc);
/* S_calc of the bottom (which = 0, HB/EB) or top (1, HT/ET) monitor plane:
 * 2*N_real complex values, forward modes then backward modes (S_calc :437-445
 * in the reference's summation order). */
int smat_deck_smatrix(const smat_deck *deck, int which, const double *HB, const double *EB, double *S);
/* The whole drop-in `FDTD input.txt` program (main :32-187): reads the deck,
 * runs on the GPU, prints the reference's report (including the |S|^2 table
 * of :182-185) to stderr; returns the process exit status. */
int smat_fdtd_main(int argc, char **argv);

/* Bytes copied host -> device and device -> host for this plan since it was
 * created: the uploads of creation, sources, schedules and states, and every
 * read-back (fields, monitors, DFT planes, overlaps, states, status words).
 * No counterpart in the reference (it has no device). */
int smat_fdtd_copy_bytes(const smat_fdtd_plan *plan, long long *h2d, long long *d2h);

/* Largest |field| over every excitation (a NaN/Inf check); *finite = 0 when a
 * non-finite value is present. */
int smat_fdtd_check_finite(smat_fdtd_plan *plan, int *finite, double *max_abs);

/* Average device time per launch (ms) of the H sweep, the E sweep and the
 * per-step DFT work (FP64: the DFT kernel; FP32: the ring flush amortised over
 * its steps), measured with CUDA events on the plan's stream over steps
 * [k_begin, k_begin+nsteps) of the schedule.  The steps are really taken. */
int smat_fdtd_time_kernels(smat_fdtd_plan *plan, int k_begin, int nsteps, double ms[3]);

/* FP32 launch configuration (smat_fdtd_autotune picks one by timing).
 *   kernel 0: two sweeps with 32 x tile_y thread blocks (1..8); z_chunk > 0
 *             runs H and E in chunks of that many planes (0: whole grid).
 *   kernel 2: two sweeps of four cells per thread (float4, L0 % 4 == 0,
 *             tile_y 1..4; the default where it applies); z_chunk as for 0;
 *             ctas_per_sm = register bound as minimum resident blocks (0 or 5:
 *             96 registers, 6, 8), or -3 for two z-planes per thread (168).
 *   kernel 6: one fused launch per step; a CTA marches tile_y whole x rows
 *             along z through z_chunk planes (0: persistent CTAs), four cells
 *             a thread, the next plane's inputs staged by cp.async;
 *             ctas_per_sm is its register bound (1..3 resident CTAs per SM);
 *             slots is the warp order (0: quads in order; 1: in blocks of a
 *             multiple of 128 threads, at least 256, the last two warps --
 *             mostly the halo row's -- trade places with the two before
 *             them, so they share the SM sub-partitions of the split quads'
 *             warps; the autotuner's choice); for plans with L0 % 4 == 0 (lossy and PEC
 *             ordinary cells, lossy split cells and metal cells run an
 *             out-of-line record update; plans with metal cells add a second,
 *             small launch per step for their stable-form E update and their
 *             monitor samples).
 * Other kernel codes are refused (SMAT_EINVAL).  Results are bit-identical
 * across configurations. */
int smat_fdtd_set_tuning(smat_fdtd_plan *plan, int kernel, int tile_y, int z_chunk, int ctas_per_sm,
                         int slots);
/* {kernel, tile_y, z_chunk, ctas_per_sm, slots} of the plan. */
int smat_fdtd_get_tuning(const smat_fdtd_plan *plan, int out[5]);
/* Autotuner: times the candidate FP32 configurations (tile rows, z chunk,
 * register bound; the fused step and the two sweeps) for nsteps steps each on this plan's
 * structure and batch, and keeps the fastest (returned in best, its time per
 * step in *best_ms; either may be NULL).  Needs the zero state (call it before
 * set_fields / run); sources and DFT sampling are off while it runs, so the
 * plan is left unchanged apart from its configuration.  FP64: no-op. */
int smat_fdtd_autotune(smat_fdtd_plan *plan, int nsteps, int best[5], double *best_ms);

/* The work partition of launch form 6, run on the host: the pieces {row
 * tile, z0, z1} (planes [z0, z1) of rows tile*tile_y ..) that CTA group gidx
 * of every excitation marches on an L1 x L2 (rows x planes) grid, with
 * z_chunk planes per item (gidx = item, row tile fastest) or persistent
 * groups (z_chunk = 0, ngroups groups).  Up to max_pieces triples into out,
 * their count in *n.  Needs no GPU: a check that the pieces of all groups
 * cover every cell exactly once (no two CTAs write one cell). */
int smat_row32_pieces(int L1, int L2, int tile_y, int z_chunk, int ngroups, int gidx, int *out, int max_pieces,
                      int *n);

/* Name, SM count and compute capability (major*10+minor) of the current device. */
int smat_device_info(char *name, int name_len, int *sm_count, int *cc);

/* Device bytes the plan holds. */
long long smat_fdtd_device_bytes(const smat_fdtd_plan *plan);

/* ---------------------------------------------------------------------------
 * Port eigenmodes of one z layer (the reference mode solver, ModeCalc/Mcalc.c).
 *
 * Media `med`: 6*L0*L1 complex values (interleaved re, im) of the layer's Med
 * file, value times metric factor, in the file's column order -- rows
 * [0, L0L1): mu00, then mu11, eps22 (the j2 = 0 columns), eps11, eps00, mu22
 * (the j2 = 1 columns), point p = l + L0*m within each row.  This is Vcomp of
 * set_V (Mcalc.c:1123-1160) before its omega scaling.  The imaginary parts
 * must be zero: the reference serves lossless port layers only (its sortXi
 * exits on complex modes, :620-626).  BoundC[2] in {-1, 0, 1} as in set_D.
 * --------------------------------------------------------------------------- */
typedef struct smat_mode_opts {
    double tol;              /* relative residual ||A x - l x|| / (rho ||x||); 0: 1e-12 */
    int degree;              /* initial Chebyshev filter degree per iteration (it grows
                                by that much every 4 iterations, up to 256, capped so
                                the top mode grows at most e^13 per pass); 0: 24 */
    int guard;               /* extra block vectors beyond nmodes; 0: max(8, nmodes/2) */
    int max_iter;            /* outer iterations; 0: 2000 */
    unsigned long long seed; /* start block; 0: fixed default */
    int precision;           /* 0: FP32 filter passes until the wanted residuals are below
                                1e-6, then FP64 (default); 1: FP64 passes throughout.
                                The Rayleigh-Ritz step and the result are FP64 either way */
} smat_mode_opts;

typedef struct smat_mode_info {
    int n_found;          /* propagating modes returned (<= nmodes) */
    int iterations;       /* outer (filter + Rayleigh-Ritz) iterations */
    int degenerate_pairs; /* mode pairs degeneXi re-orthogonalised */
    int block;            /* block size used */
    long long matvecs;    /* applications of mbb*maa to one vector (FP32 and FP64) */
    double max_residual;  /* largest relative residual among returned modes */
    double spectral_radius;
    double ms;            /* wall time of the call */
    long long matvecs_fp32; /* of matvecs, those done in FP32 filter passes */
} smat_mode_info;

/* Replaces calc_Xi (Mcalc.c:256-347) for the propagating part of the spectrum:
 * the nmodes eigenpairs of mbb*maa with the largest eigenvalues (those with a
 * positive eigenvalue; fewer when the layer has fewer propagating modes),
 * turned into Mcalc's outputs for those modes.  theta: 2*nmodes complex,
 * theta[j] and theta[j + nmodes] = -theta[j] (makeXi :651-654), descending.
 * Xi: (4*L0*L1) x (2*nmodes) complex, column-major -- forward column j =
 * [e^{-i theta/2} H; E], backward column nmodes + j = [e^{+i theta/2} H; -E]
 * with H rows (H0 of all points, H1 of all points), E = maa H / eiSin
 * (makeE :731-757), power-normalised (normXi :529-561) and degenerate modes
 * re-orthogonalised (degeneXi :417-467).  The sign of each eigenvector is
 * fixed by making its largest H entry positive (dgeev leaves it open).
 * Columns past info->n_found are zero.  opts and info may be NULL. */
int smat_mode_solve(int L0, int L1, const int BoundC[2], double omega, const double *med, int nmodes,
                    const smat_mode_opts *opts, double *theta, double *Xi, smat_mode_info *info);

/* No counterpart in the reference: applies maa (which = 0), mbb (1) or
 * mbb*maa (2) of the layer to the m columns of X (2*L0*L1 doubles each) on
 * the GPU, into Y.  The stencils the solver uses, exposed for checking them
 * against Mcalc's dense set_M matrices. */
int smat_mode_apply(int L0, int L1, const int BoundC[2], double omega, const double *med, int which, int m,
                    const double *X, double *Y);

/* No counterpart in the reference: the host eigen solver of the mode solver's
 * Rayleigh-Ritz step (complex Schur form by shifted QR), for testing.  B: m x m
 * complex row-major; w: m eigenvalues; V: m x m, eigenvector k in column k
 * (unit 2-norm).  Host only, no GPU needed. */
int smat_mode_small_eig(int m, const double *B, double *w, double *V);

/* ---------------------------------------------------------------------------
 * Frequency-domain S matrix by layer transfer (the reference's Smat/Scalc.c).
 * --------------------------------------------------------------------------- */
typedef struct smat_scalc_info {
    double ms;         /* wall time of the call */
    int solves;        /* dense eliminations (inv_process) performed */
    double unitarity;  /* ||S^H S - 1||_F   (check_Smat :885-912) */
    double transpose;  /* ||S - S^T||_F */
} smat_scalc_info;

/* Scalc's main (:74-96): the S matrix between the bottom port layer iB and the
 * top port layer iT.  meds: nlayers = iT - iB + 1 layers in z order, each
 * 6*L0*L1 complex Med values as set_V reads them (the port layers must be
 * lossless, inner layers may be lossy); XiB / XiT: the full mode matrices of
 * the two port layers, (4*L0*L1) x (4*L0*L1) complex column-major as Mcalc's
 * Xi file holds them (column j forward mode j, column j + 2*L0*L1 backward);
 * nB / nT: their N_real.  both_ways = 0 computes the first nB columns only
 * (the forward pass).  S: (nB+nT)^2 complex, column-major, Smat_calc's
 * layout.  Dense in 2*L0*L1, as the reference: cross-sections up to a few
 * thousand unknowns. */
int smat_scalc(int L0, int L1, const int BoundC[2], double omega, int nlayers, const double *meds,
               const double *XiB, int nB, const double *XiT, int nT, int both_ways, double *S,
               smat_scalc_info *info);

/* No counterpart in the reference: the GPU LU solve behind smat_scalc (zgesv
 * semantics) on host arrays, for testing.  A: n x n, B and X: n x nrhs, all
 * complex column-major; *info = first zero pivot (1-based) or 0. */
int smat_zgesv(int n, int nrhs, const double *A, const double *B, double *X, int *info);

/* Replaces the zgemm_ calls of Scalc's inv_process (Smat/Scalc.c:316-400) as
 * smat_scalc runs them: C += alpha * A * B on the GPU, on host arrays, for
 * testing.  A: m x k (lda), B: k x n (ldb), C: m x n (ldc), complex
 * column-major; alpha: one complex (re, im).  mode 1: FP64-accurate products
 * on the tensor cores (bf16 slices of the operands, Ozaki scheme, 7 slices);
 * mode 0: the FP64 multiply-add kernel. */
int smat_zgemm(int mode, int m, int n, int k, const double *alpha, const double *A, int lda, const double *B, int ldb,
               double *C, int ldc);

/* No counterpart in the reference: the device time of one smat_zgemm product
 * of these sizes (operands seeded on the device, CUDA events around reps
 * calls after a warm-up), in *ms per call. */
int smat_zgemm_time(int mode, int m, int n, int k, int reps, double *ms);

/* No counterpart in the reference: the failure path of the tensor-core
 * product's bounded waits, for testing.  Runs one small product (128 x 32,
 * inner 32) in which one slice pair is never loaded and the waits give up
 * after a few thousand polls; *flag receives the error code the kernel
 * records (1: gave up waiting for its operands), the device stays usable.
 * Returns 0 when the call itself completed. */
int smat_zgemm_wait_test(int *flag);

/* No counterpart in the reference: how smat_scalc and smat_zgesv multiply
 * (process-wide): 1 (the default) the tensor-core products of smat_zgemm
 * mode 1, where the device gives them their shared memory; 0 the FP64
 * multiply-add kernel. */
int smat_dense_mode(int mode);

/* The drop-in S-matrix program: `Scalc input.txt` reads the keys, Med layers,
 * Mode and Xi files Scalc reads (Smat/Scalc.c main :27-96) and writes
 * <prefix>_Smatrix.dat in Out_Smat's format (:113-140); returns the exit status. */
int smat_scalc_main(int argc, char **argv);

#ifdef __cplusplus
}
#endif
#endif
