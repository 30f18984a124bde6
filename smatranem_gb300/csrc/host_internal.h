/* Internal host-side helpers shared by the C and CUDA translation units. */
#ifndef SMATRAN_HOST_INTERNAL_H
#define SMATRAN_HOST_INTERNAL_H

#ifdef __cplusplus
extern "C" {
#endif

/* Records a printf-style message for smat_last_error() and returns code. */
int smat_fail(int code, const char *fmt, ...);
void smat_clear_error(void);

/* exp(i*phi) table of main :93-99, 2*N complex into out (4*N doubles). */
int host_expn(int N, double *out);
/* The reference CW run as a schedule: src 6 doubles per step, phase 4 doubles
 * per step, stop-period*N steps (main :153-167). */
int host_cw_schedule(int N, const int time_period[3], double *src, double *phase);

/* Host worker threads for a loop over `work` cells: SMATRAN_HOST_THREADS when it
 * is set to 1..HOST_MAX_THREADS, else one per online core (at most 16) for a
 * million cells or more, else 1. */
#define HOST_MAX_THREADS 64
int host_threads(long long work);
/* fn(ctx, lo, hi) over [0, n) cut into nt contiguous ranges, range 0 on the
 * calling thread; returns when all have run.  A range whose thread cannot be
 * created runs on the calling thread afterwards. */
typedef void (*host_range_fn)(void *ctx, long long lo, long long hi);
void host_parallel_for(long long n, int nt, host_range_fn fn, void *ctx);

struct smat_fdtd_plan;
int smat_fdtd_dft_count(const struct smat_fdtd_plan *plan, int *nfreq, int *nplanes);

#ifdef __cplusplus
}
#endif
#endif
