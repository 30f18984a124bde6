/*
 * Reading the FDTD's input deck -- input.txt and the Data/ files the SMatrAnEM
 * mesher chain writes -- and the drop-in `FDTD` program built on it.
 *
 * File formats are the reference's (FDTDcalc/FDTDsplitfieldMetal.c): the same
 * keys, the same sscanf conversions and the same consistency checks, so a deck
 * the reference accepts is read to the same numbers and a deck it rejects is
 * rejected here with an error code instead of exit().  Differences that only
 * cost the reference time: tilde-Xi and the incident column are read from the
 * first max(N_real, |inci_mode|) column blocks of each Xi file, once, instead
 * of the whole (4*L0*L1)^2 matrix up to four times.
 */
#define _POSIX_C_SOURCE 200809L /* stat's nanosecond mtime, for the deck cache */

#include "host_internal.h"
#include "smatran_fdtd.h"

#include <complex.h>
#include <stdint.h>
#include <sys/stat.h>
#include <unistd.h>
#include <ctype.h>
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define BUF 1024                                                       /* FDTDcalc/constant.h:5 */
#define TWO_PI_LD (2.0L * 3.1415926535897932384626433832795028841971L) /* constant.h:13-15 */

struct smat_deck {
    int L[4];
    int iBc[3];
    int tp[3];
    int iB, iT, iI, inci_mode;
    double dt_factor, omega, wavelength, k0, min_dt;
    char prefix[BUF], target[2][BUF], inci_point[BUF];
    int precision; /* extra key "FDTD_GPU: precision = FP32" (ignored by the reference) */
    int use_cache;  /* extra key "FDTD_GPU: cache = y": keep a binary copy of the parsed deck */
    int solve_modes; /* extra key "FDTD_GPU: modes = solve[, nmodes = K]": port modes from the
                        GPU mode solver on the monitor layers instead of the Mode / Xi files */
    int nmodes_req;  /* K: at most this many propagating modes per side (default 64) */
    int from_cache; /* this load came from that copy */
    double complex *mu, *epsi;
    double complex *Hinc, *Einc;
    int nreal[2];                /* bottom, top */
    int ncols[2];                /* tilde-Xi columns kept per side: 2*nreal (forward + backward) */
    double complex *tilxi[2];    /* [ncols][4*L0*L1], reported columns c < nreal and c + 2L0L1 */
    double xi_check;             /* ||tilXi^H Xi - I||_F of the incident side, or -1 if not computed */
    int changed_iT;
};

/* ---- small text helpers: input_file0 :757-817 ------------------------------ */

static void strip_leading_space(char *a)
{
    size_t i = 0;
    while (a[i] && isspace((unsigned char)a[i])) i++;
    if (i) memmove(a, a + i, strlen(a + i) + 1);
}

static void cut_at_comma(char *a)
{
    char *c = strchr(a, ',');
    if (c) *c = '\0';
}

/* "B<k>" (bottom outer layer k), "T<k>" (top outer layer), "<k>" (scatterer
 * layer): the z index of a plane (num_u2 :703-710) */
static int plane_index(const int L[4], const char *s)
{
    int k = -1;
    if (s[0] == 'B') sscanf(s + 1, "%d", &k);
    else if (s[0] == 'T') {
        sscanf(s + 1, "%d", &k);
        k += L[2] - L[3];
    } else {
        sscanf(s, "%d", &k);
        k += L[3];
    }
    return k;
}

/* layer file of z index istep (matdata_file :714-720) */
static void layer_file(const char *prefix, const int L[4], int istep, char *out)
{
    if (istep < L[3]) snprintf(out, BUF, "%s_MedB%d.dat", prefix, istep);
    else if (istep < L[2] - L[3]) snprintf(out, BUF, "%s_Med%d.dat", prefix, istep - L[3]);
    else snprintf(out, BUF, "%s_MedT%d.dat", prefix, istep - (L[2] - L[3]));
}

static int read_input(smat_deck *d, const char *path)
{
    FILE *f = fopen(path, "r");
    if (!f) return smat_fail(SMAT_EINVAL, "open error!: open input-file0! (%s)", path);
    char buf[BUF];
    int seen = 0;
    d->precision = SMAT_FP64;
    while (fgets(buf, sizeof buf, f)) {
        strip_leading_space(buf);
        if (!(seen & 1) && strncmp(buf, "Prefix", 6) == 0 && sscanf(buf, "%*[^=] %*[=] %s", d->prefix) == 1) {
            cut_at_comma(d->prefix);
            seen |= 1;
        } else if (!(seen & 2) && strncmp(buf, "BoundaryCondition", 17) == 0 &&
                   sscanf(buf, "%*[^=] %*[=] %d %*[^=] %*[=] %d %*[^=] %*[=] %d", &d->iBc[0], &d->iBc[1],
                          &d->iBc[2]) == 3) {
            seen |= 2;
        } else if (!(seen & 4) && strncmp(buf, "ModeP", 5) == 0 &&
                   sscanf(buf, "%*[^=] %*[=] %*[^=] %*[=] %*[^=] %*[=] %s", d->target[0]) == 1) {
            cut_at_comma(d->target[0]);
            if (sscanf(buf, "%*[^=] %*[=] %*[^=] %*[=] %*[^=] %*[=] %*[^=] %*[=] %s", d->target[1]) != 1)
                sscanf(d->target[0], "%s", d->target[1]);
            else cut_at_comma(d->target[1]);
            seen |= 4;
        } else if (strncmp(buf, "FDTD_GPU", 8) == 0) {
            if (strstr(buf, "FP32") || strstr(buf, "fp32")) d->precision = SMAT_FP32;
            const char *c = strstr(buf, "cache");
            if (c && (c = strchr(c, '=')) != NULL) {
                while (*++c == ' ')
                    ;
                d->use_cache = *c == 'y' || *c == 'Y' || *c == '1';
            }
            const char *m = strstr(buf, "modes");
            if (m && (m = strchr(m, '=')) != NULL) {
                while (*++m == ' ')
                    ;
                d->solve_modes = strncmp(m, "solve", 5) == 0;
            }
            const char *k = strstr(buf, "nmodes");
            if (k && (k = strchr(k, '=')) != NULL) d->nmodes_req = atoi(k + 1);
        } else if (!(seen & 8) && strncmp(buf, "FDTD", 4) == 0 &&
                   sscanf(buf,
                          "%*[^=] %*[=] %d %*[^=] %*[=] %d %*[^=] %*[=] %d %*[^=] %*[=] %s %*[^=] %*[=] %d "
                          "%*[^=] %*[=] %lf",
                          &d->tp[0], &d->tp[1], &d->tp[2], d->inci_point, &d->inci_mode, &d->dt_factor) == 6) {
            cut_at_comma(d->inci_point);
            seen |= 8;
        }
    }
    fclose(f);
    if (seen != 15) return smat_fail(SMAT_EINVAL, "4 control commands cannot be read in input_file0!");
    return SMAT_OK;
}

/* L, omega from <prefix>_Med0.dat and the Omega check of _bMode.dat (input_Lf :724-752) */
static int read_geometry(smat_deck *d)
{
    char name[BUF + 32], buf[BUF];
    snprintf(name, sizeof name, "%s_Med0.dat", d->prefix);
    FILE *f = fopen(name, "r");
    if (!f) return smat_fail(SMAT_EINVAL, "open error for %s", name);
    int n = -3;
    while (n < 0 && fgets(buf, sizeof buf, f)) {
        if (sscanf(buf, "%*[^<] %*[<] %d %*[^<] %*[<] %d %*[^<] %*[<] %d %*[^<] %*[<] %*[^=] %*[=] %d", &d->L[0],
                   &d->L[1], &d->L[2], &d->L[3]) == 4)
            n++;
        else if (strncmp(buf, "# wavelength", 12) == 0 && sscanf(buf, "%*[^=] %*[=] %lf", &d->wavelength) == 1)
            n++;
        else if (strncmp(buf, "# k_0", 5) == 0 && sscanf(buf, "%*[^=] %*[=] %*[^=] %*[=] %lf", &d->k0) == 1)
            n++;
    }
    fclose(f);
    if (n < 0) return smat_fail(SMAT_EINVAL, "L,M,N,N_outer can not be read at Scatterer @ input_file0!");
    d->omega = TWO_PI_LD / (d->wavelength * d->k0);
    if (d->L[0] <= 0 || d->L[1] <= 0 || d->L[2] <= 0 || d->L[3] < 0)
        return smat_fail(SMAT_EINVAL, "bad lattice numbers %d %d %d %d", d->L[0], d->L[1], d->L[2], d->L[3]);
    if (d->solve_modes) return SMAT_OK; /* modes computed at this omega: no Mode file to check against */
    snprintf(name, sizeof name, "%s_bMode.dat", d->prefix);
    f = fopen(name, "r");
    if (!f) return smat_fail(SMAT_EINVAL, "open error for %s", name);
    double om = 0;
    n = -1;
    while (n < 0 && fgets(buf, sizeof buf, f))
        if (strncmp(buf, "# Omega", 7) == 0 && sscanf(buf, "%*[^=] %*[=] %lf", &om) == 1) n++;
    fclose(f);
    if (n != 0) return smat_fail(SMAT_EINVAL, "Omega can not be read in input_Lf!");
    if (d->omega != om) return smat_fail(SMAT_EINVAL, "Omega = %.5e != %.5e in input_Lf!", d->omega, om);
    if (d->L[0] <= 0 || d->L[1] <= 0 || d->L[2] <= 0 || d->L[3] < 0)
        return smat_fail(SMAT_EINVAL, "bad lattice numbers %d %d %d %d", d->L[0], d->L[1], d->L[2], d->L[3]);
    return SMAT_OK;
}

/* one Med layer (input_data :665-699): header "min Dt^2", then 2*L0*L1 lines
 * "l m j2 Re Im Re Im Re Im fx fx fx" in (j2, l, m) order; j2 = 0 carries
 * (mu00, mu11, epsi22), j2 = 1 (epsi11, epsi00, mu22), each value (Re+iIm)*fx */
static int read_layer(const char *name, const int L[4], double *min_sqdt, double complex *mu, double complex *ep)
{
    FILE *f = fopen(name, "r");
    if (!f) return smat_fail(SMAT_EINVAL, "open error for %s", name);
    char buf[BUF];
    int j0 = 0, j1 = 0, j2 = 0, head = -1, count = 0;
    while (fgets(buf, sizeof buf, f)) {
        if (strncmp(buf, "# l <", 5) == 0 &&
            sscanf(buf, "%*[^<] %*[<] %*[^<] %*[<] %*[^<] %*[<] %*[^<] %*[<] %*[^=] %*[=] %*[^=] %*[=] %*[^=] %*[=] %lf",
                   min_sqdt) == 1)
            head++;
        int jl, jm, jn;
        double r0, i0, r1, i1, r2, i2, f0, f1, f2;
        if (sscanf(buf, "%d %d %d %lf %lf %lf %lf %lf %lf %lf %lf %lf", &jl, &jm, &jn, &r0, &i0, &r1, &i1, &r2, &i2,
                   &f0, &f1, &f2) == 12) {
            if (jl != j0 || jm != j1 || jn != j2 || j1 >= L[1]) {
                fclose(f);
                return smat_fail(SMAT_EINVAL, "Data cannot be read in input_data2! (%s: %s)", name, buf);
            }
            const long p = 3L * (j0 + (long)L[0] * j1);
            if (j2 == 0) {
                mu[0 + p] = (r0 + I * i0) * f0;
                mu[1 + p] = (r1 + I * i1) * f1;
                ep[2 + p] = (r2 + I * i2) * f2;
            } else {
                ep[1 + p] = (r0 + I * i0) * f0;
                ep[0 + p] = (r1 + I * i1) * f1;
                mu[2 + p] = (r2 + I * i2) * f2;
            }
            if (++j2 == 2) {
                j2 = 0;
                if (++j0 == L[0]) {
                    j0 = 0;
                    j1++;
                }
            }
            count++;
        }
    }
    fclose(f);
    if (head < 0) return smat_fail(SMAT_EINVAL, "min_sqDt can not be read in input_data! (%s)", name);
    if (count != 2 * L[0] * L[1])
        return smat_fail(SMAT_EINVAL, "j_count2 = %d != %d in input_data! (%s)", count, 2 * L[0] * L[1], name);
    return SMAT_OK;
}

/* N_real of a Mode file (get_RealNum :632-661) */
static int read_nreal(const char *name, const int L[4], int *nreal)
{
    FILE *f = fopen(name, "r");
    if (!f) return smat_fail(SMAT_EINVAL, "open error for %s", name);
    char buf[BUF];
    int heads = -1, nr = 0, nc = 0, count = 0;
    while (fgets(buf, sizeof buf, f)) {
        int a, b;
        double x0, y0, x1, y1;
        if (strncmp(buf, "# Eigen-value", 13) == 0 && sscanf(buf, "%*[^=] %*[=] %d %*[^=] %*[=] %d", &nr, &nc) == 2)
            heads++;
        else if (strncmp(buf, "theta[", 6) == 0 &&
                 sscanf(buf, "%*[^[] %*[[] %d %*[^(] %*[(] %lf %*[,] %lf %*[^[] %*[[] %d %*[^(] %*[(] %lf %*[,] %lf",
                        &a, &x0, &y0, &b, &x1, &y1) == 6) {
            if (a != count) {
                fclose(f);
                return smat_fail(SMAT_EINVAL, "theta cannot be read in get_RealNum05! (%s)", name);
            }
            count++;
        }
    }
    fclose(f);
    if (heads != 0 || nr + nc != 2 * L[0] * L[1] || count != 2 * L[0] * L[1])
        return smat_fail(SMAT_EINVAL, "RealNum05 cannot be read in get_RealNum05! (%s)", name);
    *nreal = nr;
    return SMAT_OK;
}

/* The first nblocks column blocks of an Xi file (set_Xi :557-594): block j holds
 * Xi columns j and j + NA as 2*NA rows of "re im re im".  Returns the blocks as
 * xi[j][row][2] complex (column j then column j + NA). */
static int read_xi_blocks(const char *name, int NA, int nblocks, double complex *xi)
{
    FILE *f = fopen(name, "r");
    if (!f) return smat_fail(SMAT_EINVAL, "open error!: open %s!", name);
    char buf[BUF];
    for (int j = 0; j < 2; j++)
        if (!fgets(buf, sizeof buf, f)) {
            fclose(f);
            return smat_fail(SMAT_EINVAL, "set_tilPhi error! (%s)", name);
        }
    for (int col = 0; col < nblocks; col++) {
        if (!fgets(buf, sizeof buf, f)) {
            fclose(f);
            return smat_fail(SMAT_EINVAL, "set_tilPhi error! (%s)", name);
        }
        int idx = -1;
        if (sscanf(buf, "%*[^[] %*[[] %d", &idx) == 1 && idx != col) {
            fclose(f);
            return smat_fail(SMAT_EINVAL, "dummyi = %d, jcolumn = %d! (%s)", idx, col, name);
        }
        for (int row = 0; row < 2 * NA; row++) {
            double a, b, c, e;
            if (!fgets(buf, sizeof buf, f) || sscanf(buf, "%lf %lf %lf %lf", &a, &b, &c, &e) != 4) {
                fclose(f);
                return smat_fail(SMAT_EINVAL, "From %s, data cannot be read at column = %d, row = %d!", name, col, row);
            }
            xi[((size_t)col * 2 * NA + row) * 2 + 0] = a + I * b;
            xi[((size_t)col * 2 * NA + row) * 2 + 1] = c + I * e;
        }
    }
    fclose(f);
    return SMAT_OK;
}

static void xi_names(const smat_deck *d, int top, char *xi, char *mode)
{
    snprintf(xi, BUF + 32, "%s_%cXi.dat", d->prefix, top ? 't' : 'b');
    snprintf(mode, BUF + 32, "%s_%cMode.dat", d->prefix, top ? 't' : 'b');
}

/* Side (0 bottom, 1 top) of a monitor plane for S_calc (:422-431). */
static int plane_side(const int L[4], int z)
{
    if (z >= 0 && z < L[3]) return 0;
    if (z >= L[2] - L[3] && z < L[2]) return 1;
    return -1;
}

/* ---- optional binary cache of a parsed deck --------------------------------
 * Text parsing dominates the reference program's run time on real decks (the
 * Med files hold 2*L0*L1 lines per layer, the Xi files (4*L0*L1)^2 numbers).
 * With "FDTD_GPU: cache = y" in input.txt the parsed arrays are kept in
 * <prefix>.smatdeck, keyed by a signature of every source file's size and
 * modification time and of the input.txt keys that select what is kept; a
 * later load with the same signature reads the binary copy instead.  The copy
 * is written to a temporary name and renamed, so a reader never sees half of
 * one. */
#define CACHE_MAGIC "SMATDECK1"

static uint64_t fnv1a(uint64_t h, const void *p, size_t n)
{
    const unsigned char *c = (const unsigned char *)p;
    for (size_t i = 0; i < n; i++) h = (h ^ c[i]) * 1099511628211ULL;
    return h;
}

static uint64_t file_sig(uint64_t h, const char *name)
{
    struct stat st;
    long long v[3] = {-1, -1, -1};
    if (stat(name, &st) == 0) {
        v[0] = (long long)st.st_size;
        v[1] = (long long)st.st_mtim.tv_sec;
        v[2] = (long long)st.st_mtim.tv_nsec;
    }
    h = fnv1a(h, name, strlen(name));
    return fnv1a(h, v, sizeof v);
}

static uint64_t deck_signature(const smat_deck *d)
{
    uint64_t h = 14695981039346656037ULL;
    h = fnv1a(h, d->prefix, strlen(d->prefix));
    h = fnv1a(h, d->target[0], strlen(d->target[0]));
    h = fnv1a(h, d->target[1], strlen(d->target[1]));
    h = fnv1a(h, d->inci_point, strlen(d->inci_point));
    h = fnv1a(h, &d->inci_mode, sizeof d->inci_mode);
    h = fnv1a(h, d->L, sizeof d->L);
    for (int z = 0; z < d->L[2]; z++) {
        char name[BUF];
        layer_file(d->prefix, d->L, z, name);
        h = file_sig(h, name);
    }
    for (int side = 0; side < 2; side++) {
        char xi[BUF + 32], mode[BUF + 32];
        xi_names(d, side, xi, mode);
        h = file_sig(h, xi);
        h = file_sig(h, mode);
    }
    return h;
}

static void cache_name(const smat_deck *d, char *out) { snprintf(out, BUF + 32, "%s.smatdeck", d->prefix); }

/* everything smat_deck_load derives from the data files */
static int cache_io(smat_deck *d, FILE *f, int writing)
{
    const long n3 = (long)d->L[0] * d->L[1] * d->L[2], pl = (long)d->L[0] * d->L[1], NA = 2 * pl;
#define IO(ptr, n)                                                                                                     \
    do {                                                                                                               \
        const size_t n_ = (size_t)(n);                                                                                 \
        if ((writing ? fwrite((ptr), sizeof *(ptr), n_, f) : fread((ptr), sizeof *(ptr), n_, f)) != n_) return -1;     \
    } while (0)
    IO(d->nreal, 2);
    IO(d->ncols, 2);
    IO(&d->iB, 1);
    IO(&d->iT, 1);
    IO(&d->iI, 1);
    IO(&d->changed_iT, 1);
    IO(&d->min_dt, 1);
    if (!writing) {
        if (d->ncols[0] < 0 || d->ncols[1] < 0 || d->ncols[0] > 2 * NA || d->ncols[1] > 2 * NA) return -1;
        d->mu = calloc(3 * n3, sizeof(double complex));
        d->epsi = calloc(3 * n3, sizeof(double complex));
        d->Hinc = calloc(2 * pl, sizeof(double complex));
        d->Einc = calloc(2 * pl, sizeof(double complex));
        for (int s = 0; s < 2; s++)
            if (d->ncols[s]) d->tilxi[s] = calloc((size_t)d->ncols[s] * 2 * NA + 1, sizeof(double complex));
        if (!d->mu || !d->epsi || !d->Hinc || !d->Einc) return -1;
        for (int s = 0; s < 2; s++)
            if (d->ncols[s] && !d->tilxi[s]) return -1;
    }
    IO(d->mu, 3 * n3);
    IO(d->epsi, 3 * n3);
    IO(d->Hinc, 2 * pl);
    IO(d->Einc, 2 * pl);
    for (int s = 0; s < 2; s++)
        if (d->ncols[s]) IO(d->tilxi[s], (size_t)d->ncols[s] * 2 * NA);
#undef IO
    return 0;
}

static int read_cache(smat_deck *d, uint64_t sig)
{
    char name[BUF + 32], magic[sizeof CACHE_MAGIC];
    cache_name(d, name);
    FILE *f = fopen(name, "rb");
    if (!f) return -1;
    uint64_t s = 0;
    int L[4];
    int rc = fread(magic, 1, sizeof magic, f) == sizeof magic && memcmp(magic, CACHE_MAGIC, sizeof magic) == 0 &&
                     fread(&s, sizeof s, 1, f) == 1 && s == sig && fread(L, sizeof L, 1, f) == 1 &&
                     memcmp(L, d->L, sizeof L) == 0
                 ? cache_io(d, f, 0)
                 : -1;
    fclose(f);
    return rc;
}

static void write_cache(smat_deck *d, uint64_t sig)
{
    char name[BUF + 32], tmp[BUF + 64];
    cache_name(d, name);
    snprintf(tmp, sizeof tmp, "%s.tmp%ld", name, (long)getpid()); /* one writer per process */
    FILE *f = fopen(tmp, "wb");
    if (!f) return; /* the cache is optional: no copy, no error */
    int ok = fwrite(CACHE_MAGIC, 1, sizeof CACHE_MAGIC, f) == sizeof CACHE_MAGIC && fwrite(&sig, sizeof sig, 1, f) == 1 &&
             fwrite(d->L, sizeof d->L, 1, f) == 1 && cache_io(d, f, 1) == 0;
    ok = (fclose(f) == 0) && ok;
    if (!ok || rename(tmp, name) != 0) remove(tmp);
}

void smat_deck_free(smat_deck *d)
{
    if (!d) return;
    free(d->mu);
    free(d->epsi);
    free(d->Hinc);
    free(d->Einc);
    free(d->tilxi[0]);
    free(d->tilxi[1]);
    free(d);
}

/* Port modes of one side from the GPU mode solver (smat_mode_solve, the
 * few-mode counterpart of ModeCalc/Mcalc.c calc_Xi) on monitor layer z: the
 * layer's Med values in Mcalc's set_V order, at most d->nmodes_req
 * propagating modes.  Fills what the Mode / Xi files would have given:
 * N_real, the tilde-Xi columns of set_tilXi (:617-619) and, on the incident
 * side, the incident sheets of set_incident (:497-510). */
static int solve_side(smat_deck *d, int side, int z, int incident)
{
    const int *L = d->L;
    const long pl = (long)L[0] * L[1], NA = 2 * pl;
    int K = d->nmodes_req > 0 ? d->nmodes_req : 64;
    if (K > 85) K = 85; /* with the solver's guard vectors the block stays within 128 */
    if (K > NA) K = (int)NA;
    const int am = abs(d->inci_mode);
    if (incident && am > K) K = am;
    double complex *med = malloc(sizeof(double complex) * 6 * pl);
    double complex *theta = malloc(sizeof(double complex) * 2 * K);
    double complex *xi = malloc(sizeof(double complex) * (size_t)2 * NA * 2 * K);
    int rc = SMAT_OK;
    if (!med || !theta || !xi) rc = smat_fail(SMAT_ENOMEM, "deck_load: out of host memory");
    if (!rc) {
        const double complex *mu = d->mu + 3 * pl * z, *ep = d->epsi + 3 * pl * z;
        for (long p = 0; p < pl; p++) {
            med[0 * pl + p] = mu[3 * p + 0];
            med[1 * pl + p] = mu[3 * p + 1];
            med[2 * pl + p] = ep[3 * p + 2];
            med[3 * pl + p] = ep[3 * p + 1];
            med[4 * pl + p] = ep[3 * p + 0];
            med[5 * pl + p] = mu[3 * p + 2];
        }
        smat_mode_info info;
        const int bc[2] = {d->iBc[0], d->iBc[1]};
        rc = smat_mode_solve(L[0], L[1], bc, d->omega, (const double *)med, K, NULL, (double *)theta, (double *)xi,
                             &info);
        if (!rc) {
            const int nr = info.n_found;
            d->nreal[side] = nr;
            if (incident && am > nr) rc = smat_fail(SMAT_EINVAL, "inci_mode = %d > %d", d->inci_mode, nr);
            d->ncols[side] = 2 * nr;
            d->tilxi[side] = calloc((size_t)2 * nr * 2 * NA + 1, sizeof(double complex));
            if (!rc && !d->tilxi[side]) rc = smat_fail(SMAT_ENOMEM, "deck_load: out of host memory");
            for (int j = 0; j < nr && !rc; j++)
                for (long row = 0; row < 2 * NA; row++) {
                    const long r = (row + NA) % (2 * NA);
                    d->tilxi[side][(size_t)j * 2 * NA + r] = xi[(size_t)j * 2 * NA + row];
                    d->tilxi[side][(size_t)(nr + j) * 2 * NA + r] = -xi[(size_t)(K + j) * 2 * NA + row];
                }
            if (!rc && incident) {
                const double complex *c = xi + (size_t)(d->inci_mode > 0 ? am - 1 : K + am - 1) * 2 * NA;
                for (long row = NA; row < 2 * NA && !rc; row++)
                    if (cimag(c[row]) != 0.) rc = smat_fail(SMAT_EINVAL, "incident wave is not real number!");
                for (long r = 0; r < pl && !rc; r++) {
                    d->Hinc[0 + 2 * r] = c[r + 0 * pl];
                    d->Hinc[1 + 2 * r] = c[r + 1 * pl];
                    d->Einc[1 + 2 * r] = -c[r + 2 * pl];
                    d->Einc[0 + 2 * r] = c[r + 3 * pl];
                }
            }
        }
    }
    free(med), free(theta), free(xi);
    return rc;
}

int smat_deck_load(const char *input_txt, smat_deck **out)
{
    smat_clear_error();
    if (!input_txt || !out) return smat_fail(SMAT_EINVAL, "deck_load: bad arguments");
    *out = NULL;
    smat_deck *d = calloc(1, sizeof *d);
    if (!d) return smat_fail(SMAT_ENOMEM, "deck_load: out of host memory");
    d->xi_check = -1;
    int rc = read_input(d, input_txt);
    if (!rc) rc = read_geometry(d);
    if (rc) {
        smat_deck_free(d);
        return rc;
    }
    uint64_t sig = 0;
    if (d->use_cache) {
        sig = deck_signature(d);
        if (read_cache(d, sig) == 0) {
            d->from_cache = 1;
            *out = d;
            return SMAT_OK;
        }
        /* no usable copy: forget what a partial read allocated, parse the text */
        free(d->mu), free(d->epsi), free(d->Hinc), free(d->Einc), free(d->tilxi[0]), free(d->tilxi[1]);
        d->mu = d->epsi = d->Hinc = d->Einc = d->tilxi[0] = d->tilxi[1] = NULL;
    }
    const int *L = d->L;
    const long n3 = (long)L[0] * L[1] * L[2], pl = (long)L[0] * L[1];
    d->mu = calloc(3 * n3, sizeof(double complex));
    d->epsi = calloc(3 * n3, sizeof(double complex));
    if (!d->mu || !d->epsi) {
        smat_deck_free(d);
        return smat_fail(SMAT_ENOMEM, "deck_load: out of host memory");
    }
    for (int z = 0; z < L[2] && !rc; z++) {
        char name[BUF];
        double sq = 0;
        layer_file(d->prefix, L, z, name);
        rc = read_layer(name, L, &sq, d->mu + 3 * pl * z, d->epsi + 3 * pl * z);
        if (!rc && (z == 0 || d->min_dt > sqrt(sq))) d->min_dt = sqrt(sq);
    }
    if (rc) {
        smat_deck_free(d);
        return rc;
    }
    d->iB = plane_index(L, d->target[0]);
    d->iT = plane_index(L, d->target[1]);
    d->iI = plane_index(L, d->inci_point);
    if (d->iB == d->iT) {
        d->iT = (L[2] - 1) - d->iB;
        d->changed_iT = 1;
    }
    if (d->iB >= d->iT) {
        const int a = d->iB, b = d->iT;
        smat_deck_free(d);
        return smat_fail(SMAT_EINVAL, "Target_B = %d is larger than or equal to Target_T = %d", a, b);
    }
    /* mode counts and the tilde-Xi columns S_calc reports, per side */
    const int NA = 2 * (int)pl;
    int need_side[2] = {0, 0};
    const int sB = plane_side(L, d->iB), sT = plane_side(L, d->iT);
    if (sB < 0 || sT < 0) {
        const int z = sB < 0 ? d->iB : d->iT;
        smat_deck_free(d);
        return smat_fail(SMAT_EINVAL, "iB or iT = %d", z);
    }
    need_side[sB] = need_side[sT] = 1;
    const int inc_side = abs(d->iB - d->iI) < abs(d->iT - d->iI) ? 0 : 1; /* set_incident :482-488 */
    need_side[inc_side] = 1;
    if (d->inci_mode == 0) {
        smat_deck_free(d);
        return smat_fail(SMAT_EINVAL, "inci_mode = 0!");
    }
    d->Hinc = calloc(2 * pl, sizeof(double complex));
    d->Einc = calloc(2 * pl, sizeof(double complex));
    for (int side = 0; side < 2 && !rc; side++) {
        if (!need_side[side]) continue;
        if (d->solve_modes) {
            rc = solve_side(d, side, side == 0 ? d->iB : d->iT, side == inc_side);
            continue;
        }
        char xi[BUF + 32], mode[BUF + 32];
        xi_names(d, side, xi, mode);
        rc = read_nreal(mode, L, &d->nreal[side]);
        if (rc) break;
        const int nr = d->nreal[side];
        int nblocks = nr;
        const int am = abs(d->inci_mode);
        if (side == inc_side) {
            if (d->inci_mode > nr) {
                rc = smat_fail(SMAT_EINVAL, "inci_mode = %d > %d", d->inci_mode, nr);
                break;
            }
            if (am > nblocks) nblocks = am;
        }
        if (nblocks > NA) nblocks = NA;
        double complex *blk = calloc((size_t)nblocks * 2 * NA * 2 + 1, sizeof(double complex));
        if (!blk) {
            rc = smat_fail(SMAT_ENOMEM, "deck_load: out of host memory");
            break;
        }
        rc = read_xi_blocks(xi, NA, nblocks, blk);
        if (!rc) {
            /* tilde-Xi (set_tilXi :598-628): for a real-mode block j < N_real,
             * tilXi[(row+NA) % 2NA, j] = first pair, tilXi[.., j+NA] = -second
             * pair; keep columns j and j+NA for j < N_real */
            d->ncols[side] = 2 * nr;
            d->tilxi[side] = calloc((size_t)2 * nr * 2 * NA + 1, sizeof(double complex));
            for (int j = 0; j < nr && d->tilxi[side]; j++)
                for (int row = 0; row < 2 * NA; row++) {
                    const int r = (row + NA) % (2 * NA);
                    d->tilxi[side][(size_t)j * 2 * NA + r] = blk[((size_t)j * 2 * NA + row) * 2 + 0];
                    d->tilxi[side][(size_t)(nr + j) * 2 * NA + r] = -(blk[((size_t)j * 2 * NA + row) * 2 + 1]);
                }
            if (side == inc_side) {
                /* the incident column (set_incident :498-509) */
                const int j = am - 1, second = d->inci_mode < 0;
                for (int row = NA; row < 2 * NA; row++)
                    if (cimag(blk[((size_t)j * 2 * NA + row) * 2 + second]) != 0.) {
                        rc = smat_fail(SMAT_EINVAL, "incident wave is not real number!");
                        break;
                    }
                for (long r = 0; r < pl && !rc; r++) {
                    const double complex *c = blk + (size_t)j * 2 * NA * 2 + second;
                    d->Hinc[0 + 2 * r] = c[2 * (r + 0 * pl)];
                    d->Hinc[1 + 2 * r] = c[2 * (r + 1 * pl)];
                    d->Einc[1 + 2 * r] = -c[2 * (r + 2 * pl)];
                    d->Einc[0 + 2 * r] = c[2 * (r + 3 * pl)];
                }
            }
        }
        free(blk);
    }
    if (rc) {
        smat_deck_free(d);
        return rc;
    }
    if (d->use_cache) write_cache(d, sig);
    *out = d;
    return SMAT_OK;
}

int smat_deck_from_cache(const smat_deck *d) { return d ? d->from_cache : 0; }

int smat_deck_info(const smat_deck *d, int L[4], int iBTIin[4], int iBc[3], int time_period[3], double *omega,
                   double *min_dt, double *dt_factor, int nreal[2])
{
    if (!d) return smat_fail(SMAT_EINVAL, "null deck");
    if (L) memcpy(L, d->L, sizeof d->L);
    if (iBTIin) {
        iBTIin[0] = d->iB;
        iBTIin[1] = d->iT;
        iBTIin[2] = d->iI;
        iBTIin[3] = d->inci_mode;
    }
    if (iBc) memcpy(iBc, d->iBc, sizeof d->iBc);
    if (time_period) memcpy(time_period, d->tp, sizeof d->tp);
    if (omega) *omega = d->omega;
    if (min_dt) *min_dt = d->min_dt;
    if (dt_factor) *dt_factor = d->dt_factor;
    if (nreal) memcpy(nreal, d->nreal, sizeof d->nreal);
    return SMAT_OK;
}

int smat_deck_arrays(const smat_deck *d, double *mu, double *epsi, double *Hinc, double *Einc)
{
    if (!d) return smat_fail(SMAT_EINVAL, "null deck");
    const size_t n3 = (size_t)d->L[0] * d->L[1] * d->L[2], pl = (size_t)d->L[0] * d->L[1];
    if (mu) memcpy(mu, d->mu, 3 * n3 * sizeof(double complex));
    if (epsi) memcpy(epsi, d->epsi, 3 * n3 * sizeof(double complex));
    if (Hinc) memcpy(Hinc, d->Hinc, 2 * pl * sizeof(double complex));
    if (Einc) memcpy(Einc, d->Einc, 2 * pl * sizeof(double complex));
    return SMAT_OK;
}

/* S = tilXi^H (HB_x, HB_y, -EB_y, EB_x) for the kept columns, in the
 * reference's summation order (S_calc :437-445) */
static void project(const smat_deck *d, int side, const double complex *HB, const double complex *EB,
                    double complex *S)
{
    const long pl = (long)d->L[0] * d->L[1], NA = 2 * pl;
    for (int c = 0; c < d->ncols[side]; c++) {
        const double complex *t = d->tilxi[side] + (size_t)c * 2 * NA;
        double complex acc = 0.;
        for (long r = 0; r < pl; r++) {
            acc += conj(t[r]) * HB[0 + 2 * r];
            acc += conj(t[r + pl]) * HB[1 + 2 * r];
            acc += conj(t[r + NA]) * (-EB[1 + 2 * r]);
            acc += conj(t[r + pl + NA]) * EB[0 + 2 * r];
        }
        S[c] = acc;
    }
}

int smat_deck_smatrix(const smat_deck *d, int which, const double *HB, const double *EB, double *S)
{
    if (!d || which < 0 || which > 1 || !HB || !EB || !S) return smat_fail(SMAT_EINVAL, "deck_smatrix: bad arguments");
    const int side = plane_side(d->L, which ? d->iT : d->iB);
    project(d, side, (const double complex *)HB, (const double complex *)EB, (double complex *)S);
    return SMAT_OK;
}

/* ---- the drop-in program (main :32-187) ------------------------------------ */

static void print_sigma(const int L[4], const double *sigma)
{
    /* the lines set_sigma prints (:868-920) */
    const char *ax[3] = {"l0", "l1", "l2"};
    const int off[3] = {0, 2 * L[0], 2 * (L[0] + L[1])};
    for (int a = 0; a < 3; a++)
        for (int j = 0; j < L[a]; j++)
            for (int h = 0; h < 2; h++)
                if (sigma[off[a] + h + 2 * j] != 0.)
                    fprintf(stderr, "%s = %d.%d, sigma = %.5e\n", ax[a], j, h ? 5 : 0, sigma[off[a] + h + 2 * j]);
}

int smat_fdtd_main(int argc, char **argv)
{
    time_t t0 = time(0);
    fprintf(stderr, "# Start time of FDTD_SpiltField = %s\n", ctime(&t0));
    if (argc != 2) {
        fprintf(stderr, "error: number of files \n");
        return EXIT_FAILURE;
    }
    if (strncmp(argv[1], "-v", 2) == 0 || strcmp(argv[1], "--version") == 0) {
        fprintf(stderr, "The '%s' creates scattering matrix column vector by FDTD on the GPU.\n", argv[0]);
        fprintf(stderr, " smatranem_gb300 split-field FDTD (sm_103a); input and output formats of SMatrAnEM FDTD.\n");
        fprintf(stderr, "There is NO warranty.\n");
        return EXIT_SUCCESS;
    }
    smat_deck *d = NULL;
    int rc = smat_deck_load(argv[1], &d);
    if (rc) {
        fprintf(stderr, "%s\n", smat_last_error());
        return EXIT_FAILURE;
    }
    const int *L = d->L;
    const long n3 = (long)L[0] * L[1] * L[2], pl = (long)L[0] * L[1];
    fprintf(stderr, "wavelength = %.5e, k_0 = %.5e\n", d->wavelength, d->k0);
    fprintf(stderr, "Ramp-period = %d, cw-period = %d, stop-period = %d\n", d->tp[0], d->tp[1], d->tp[2]);
    fprintf(stderr, "Dt_factor = %.5e, split field impl. does not use stable_factor.\n", d->dt_factor);
    double *sigma = calloc(2 * (L[0] + L[1] + L[2]), sizeof(double));
    double *HB = calloc(4 * pl, sizeof(double)), *EB = calloc(4 * pl, sizeof(double));
    double *HT = calloc(4 * pl, sizeof(double)), *ET = calloc(4 * pl, sizeof(double));
    double complex *SB = calloc((size_t)2 * d->ncols[0] + 2 * d->ncols[1] + 2, sizeof(double complex));
    smat_fdtd_plan *plan = NULL;
    int status = EXIT_FAILURE;
    if (!sigma || !HB || !EB || !HT || !ET || !SB) {
        fprintf(stderr, "out of host memory\n");
        goto done;
    }
    rc = smat_set_sigma(L, (const double *)d->mu, (const double *)d->epsi, sigma);
    if (rc) goto fail;
    print_sigma(L, sigma);
    rc = smat_remove_sigma(L, (double *)d->mu, (double *)d->epsi, sigma);
    if (rc) goto fail;
    if (d->changed_iT) fprintf(stderr, "Change iT because iT = iB\n");
    fprintf(stderr, "Start = %d for %s, Incident point = %d for %s, Incident mode = %+d, Target_T = %d for %s\n",
            d->iB, d->target[0], d->iI, d->inci_point, d->inci_mode, d->iT, d->target[1]);
    int N = 0;
    double iR = 0, iI = 0;
    rc = smat_set_tau(d->omega, d->min_dt / d->dt_factor, &N, &iR, &iI);
    if (rc) goto fail;
    {
        const double dphi = TWO_PI_LD / ((double)N);
        const double dt = dphi / d->omega;
        fprintf(stderr, "omega = %.5e, min_Dt = %.5e, N_2pi = %d, Dt = %.5e, tau_R = %.5e, tau_I = %.5e\n", d->omega,
                d->min_dt / d->dt_factor, N, dt, 1. / iR, 1. / iI);
    }
    smat_fdtd_desc desc;
    memset(&desc, 0, sizeof desc);
    memcpy(desc.L, L, sizeof desc.L);
    memcpy(desc.iBc, d->iBc, sizeof desc.iBc);
    desc.iBTIin[0] = d->iB;
    desc.iBTIin[1] = d->iT;
    desc.iBTIin[2] = d->iI;
    desc.iBTIin[3] = d->inci_mode;
    desc.invtau_R = iR;
    desc.invtau_I = iI;
    desc.mu = (const double *)d->mu;
    desc.epsi = (const double *)d->epsi;
    desc.sigma = sigma;
    desc.precision = d->precision;
    desc.batch = 1;
    {
        /* the cell census the reference prints (:105) */
        char *cont = malloc(n3);
        int *addr = malloc(n3 * sizeof(int));
        int lnotn = 0;
        if (!cont || !addr) {
            free(cont);
            free(addr);
            fprintf(stderr, "out of host memory\n");
            goto done;
        }
        rc = smat_set_address(L, sigma, (const double *)d->mu, (const double *)d->epsi, cont, &lnotn, addr);
        free(cont);
        free(addr);
        if (rc) goto fail;
        fprintf(stderr, "L3d = %ld, Lnotn = %d\n", n3, lnotn);
    }
    rc = smat_fdtd_create(&desc, NULL, &plan);
    /* FP32: pick the launch form on the zero state (every form gives the same bits) */
    if (!rc && d->precision == SMAT_FP32) rc = smat_fdtd_autotune(plan, 4, NULL, NULL);
    if (!rc) rc = smat_fdtd_set_incident(plan, 0, (const double *)d->Hinc, (const double *)d->Einc);
    if (!rc) rc = smat_fdtd_set_cw_schedule(plan, N, d->tp);
    if (!rc) rc = smat_fdtd_run(plan, 0, d->tp[2] * N);
    if (!rc) rc = smat_fdtd_sync(plan);
    if (!rc) rc = smat_fdtd_get_monitor(plan, 0, HB, EB, HT, ET);
    if (rc) goto fail;
    {
        /* envelope normalisation check of the loop (:159-168) */
        double s00 = 0., s05 = 0.;
        for (int jp = 0; jp < d->tp[2]; jp++)
            for (int jt = 0; jt < N; jt++) {
                s00 += smat_set_env(N, d->tp, 0, (jt + 1), jp);
                s05 += smat_set_env(N, d->tp, 1, jt, jp);
            }
        fprintf(stderr, "sum00 = %.5e, sum05 = %.5e\n", s00, s05);
    }
    fprintf(stderr, "Bc[0] = %d, Bc[1] = %d, Bc[2] = %d\n", d->iBc[0], d->iBc[1], d->iBc[2]);
    {
        double complex *ST = SB + d->ncols[0] + 1;
        smat_deck_smatrix(d, 0, HB, EB, (double *)SB);
        smat_deck_smatrix(d, 1, HT, ET, (double *)ST);
        const int sB = plane_side(L, d->iB), sT = plane_side(L, d->iT);
        const int nB = d->nreal[sB], nT = d->nreal[sT];
        fprintf(stderr, "Bottom |S_(m,%+d)|^2 :\n", d->inci_mode);
        for (int m = 0; m < nB; m++)
            fprintf(stderr, "%+d, %.20e, %+d, %.20e\n", m + 1, creal(conj(SB[m]) * SB[m]), -(m + 1),
                    creal(conj(SB[m + nB]) * SB[m + nB]));
        fprintf(stderr, "Top |S_(m,%+d)|^2 :\n", d->inci_mode);
        for (int m = 0; m < nT; m++)
            fprintf(stderr, "%+d, %.20e, %+d, %.20e\n", m + 1, creal(conj(ST[m]) * ST[m]), -(m + 1),
                    creal(conj(ST[m + nT]) * ST[m + nT]));
    }
    status = EXIT_SUCCESS;
    goto done;
fail:
    fprintf(stderr, "%s\n", smat_last_error());
done:
    smat_fdtd_destroy(plan);
    free(sigma);
    free(HB);
    free(EB);
    free(HT);
    free(ET);
    free(SB);
    smat_deck_free(d);
    return status;
}

/* ---- the drop-in S-matrix program (Smat/Scalc.c main :27-96) ---------------- */

/* input_file0 of Scalc (:657-686): Prefix, BoundaryCondition (B0, B1), ModeP's
 * two targets, Smatrix (both-ways, LAPACK solver) */
static int scalc_input(const char *path, char *prefix, int bc[2], char target[2][BUF], char *both, char *solv)
{
    FILE *f = fopen(path, "r");
    if (!f) return smat_fail(SMAT_EINVAL, "open error!: open input-file0!");
    char buf[BUF];
    int seen = 0;
    while (fgets(buf, sizeof buf, f) && seen != 15) {
        strip_leading_space(buf);
        if (!(seen & 1) && strncmp(buf, "Prefix", 6) == 0 && sscanf(buf, "%*[^=] %*[=] %s", prefix) == 1) {
            cut_at_comma(prefix);
            seen |= 1;
        } else if (!(seen & 2) && strncmp(buf, "BoundaryCondition", 17) == 0 &&
                   sscanf(buf, "%*[^=] %*[=] %d %*[^=] %*[=] %d", &bc[0], &bc[1]) == 2) {
            seen |= 2;
        } else if (!(seen & 4) && strncmp(buf, "ModeP", 5) == 0 &&
                   sscanf(buf, "%*[^=] %*[=] %*[^=] %*[=] %*[^=] %*[=] %s", target[0]) == 1) {
            cut_at_comma(target[0]);
            if (sscanf(buf, "%*[^=] %*[=] %*[^=] %*[=] %*[^=] %*[=] %*[^=] %*[=] %s", target[1]) != 1)
                sscanf(target[0], "%s", target[1]);
            else cut_at_comma(target[1]);
            seen |= 4;
        } else if (!(seen & 8) && strncmp(buf, "Smatrix", 7) == 0 &&
                   sscanf(buf, "%*[^=] %*[=] %s %*[^=] %*[=] %s", both, solv) == 2) {
            cut_at_comma(both);
            cut_at_comma(solv);
            seen |= 8;
        }
    }
    fclose(f);
    if (seen != 15) return smat_fail(SMAT_EINVAL, "4 control commands cannot be read in input_file1!");
    return SMAT_OK;
}

/* N_real and omega of a Mode file (get_RealNum05omega :599-626) */
static int scalc_mode_file(const char *name, const int L[4], int *nreal, double *omega)
{
    FILE *f = fopen(name, "r");
    if (!f) return smat_fail(SMAT_EINVAL, "open error for %s", name);
    char buf[BUF];
    int need = 2, nc = 0;
    while (need > 0 && fgets(buf, sizeof buf, f)) {
        if (strncmp(buf, "# Omega", 7) == 0 && sscanf(buf, "%*[^=] %*[=] %lf", omega) == 1) need--;
        if (strncmp(buf, "# Eigen-value", 13) == 0 && sscanf(buf, "%*[^=] %*[=] %d %*[^=] %*[=] %d", nreal, &nc) == 2)
            need--;
    }
    fclose(f);
    if (need != 0 || *nreal + nc != 2 * L[0] * L[1])
        return smat_fail(SMAT_EINVAL, "RealNum05 cannot be read in get_RealNum05! (%s)", name);
    return SMAT_OK;
}

/* a whole Xi file as the (2NA x 2NA) column-major mode matrix */
static int scalc_xi(const char *name, int NA, double complex **out)
{
    double complex *blk = malloc(sizeof(double complex) * (size_t)NA * 2 * NA * 2);
    double complex *xi = malloc(sizeof(double complex) * (size_t)2 * NA * 2 * NA);
    if (!blk || !xi) {
        free(blk), free(xi);
        return smat_fail(SMAT_ENOMEM, "Scalc: out of host memory for %s", name);
    }
    int rc = read_xi_blocks(name, NA, NA, blk);
    for (long j = 0; j < NA && !rc; j++)
        for (long r = 0; r < 2 * NA; r++) {
            xi[r + 2 * NA * j] = blk[(j * 2 * NA + r) * 2 + 0];
            xi[r + 2 * NA * (j + NA)] = blk[(j * 2 * NA + r) * 2 + 1];
        }
    free(blk);
    if (rc) {
        free(xi);
        return rc;
    }
    *out = xi;
    return SMAT_OK;
}

int smat_scalc_main(int argc, char **argv)
{
    time_t t_ini = time(0);
    fprintf(stderr, "# Start time of mode calculation = %s\n", ctime(&t_ini));
    if (argc != 2) {
        fprintf(stderr, "error: number of files \n");
        return EXIT_FAILURE;
    }
    if (strncmp(argv[1], "-v", 2) == 0 || strcmp(argv[1], "--version") == 0) {
        fprintf(stderr, "The '%s' creates scattering matrix by layer transfer on the GPU.\n", argv[0]);
        fprintf(stderr, " smatranem_gb300 (sm_103a); input and output formats of SMatrAnEM Scalc.\n");
        fprintf(stderr, "There is NO warranty.\n");
        return EXIT_SUCCESS;
    }
    char prefix[BUF], target[2][BUF], both[BUF], solv[BUF];
    int bc[2], L[4] = {0, 0, 0, 0};
    int rc = scalc_input(argv[1], prefix, bc, target, both, solv);
    double complex *meds = NULL, *xiB = NULL, *xiT = NULL, *S = NULL, *mu = NULL, *ep = NULL;
    if (!rc) { /* input_file1 :643-653 */
        char name[2 * BUF + 32], buf[BUF];
        snprintf(name, sizeof name, "%s_Med%s.dat", prefix, target[0]);
        FILE *f = fopen(name, "r");
        if (!f) rc = smat_fail(SMAT_EINVAL, "open error!: open input-file1!");
        int got = 0;
        while (!rc && !got && fgets(buf, sizeof buf, f))
            if (strncmp(buf, "# l <", 5) == 0 &&
                sscanf(buf, "%*[^<] %*[<] %d %*[^<] %*[<] %d %*[^<] %*[<] %d %*[^=] %*[=] %d", &L[0], &L[1], &L[2],
                       &L[3]) == 4)
                got = 1;
        if (f) fclose(f);
        if (!rc && !got) rc = smat_fail(SMAT_EINVAL, "L[4] cannot be read in input_file1!");
    }
    int iB = 0, iT = 0, nreal[2] = {0, 0};
    double omega = 0;
    const int same = !rc && strcmp(target[0], target[1]) == 0;
    if (!rc) {
        iB = plane_index(L, target[0]);
        iT = plane_index(L, target[1]);
        if (iB == iT) {
            iT = (L[2] - 1) - iB;
            fprintf(stderr, "The 2nd target ' %s ' is the same as the 1st, and iT is changed to %d\n", target[1], iT);
        }
        if (iB >= iT)
            rc = smat_fail(SMAT_EINVAL, "Target_B = %d for %s is larger than or equal to Target_T = %d for %s", iB,
                           target[0], iT, target[1]);
        else fprintf(stderr, "Target_B = %d for %s, Target_T = %d for %s\n", iB, target[0], iT, target[1]);
    }
    for (int side = 0; side < (same ? 1 : 2) && !rc; side++) {
        char name[BUF + 32];
        double om = 0;
        snprintf(name, sizeof name, "%s_%cMode.dat", prefix, side ? 't' : 'b');
        rc = scalc_mode_file(name, L, &nreal[side], &om);
        if (!rc) fprintf(stderr, "RealNum05 for %s = %d\n", name, nreal[side]);
        if (!rc && side == 1 && om != omega)
            rc = smat_fail(SMAT_EINVAL, "Top omega = %.5e != Bottom omega = %.5e", om, omega);
        omega = om;
    }
    if (!rc && same) nreal[1] = nreal[0];
    if (!rc) fprintf(stderr, "Omega = k/k0 = %.20e\n", omega);
    const long pl = (long)L[0] * L[1];
    const int NA = 2 * (int)pl, nl = iT - iB + 1;
    if (!rc) { /* the layers iB..iT in Mcalc's set_V order */
        meds = malloc(sizeof(double complex) * 6 * pl * (nl > 0 ? nl : 1));
        mu = malloc(sizeof(double complex) * 3 * pl);
        ep = malloc(sizeof(double complex) * 3 * pl);
        if (!meds || !mu || !ep) rc = smat_fail(SMAT_ENOMEM, "Scalc: out of host memory");
        for (int z = iB; z <= iT && !rc; z++) {
            char name[BUF];
            double sq;
            layer_file(prefix, L, z, name);
            rc = read_layer(name, L, &sq, mu, ep);
            double complex *m = meds + 6 * pl * (z - iB);
            for (long p = 0; p < pl && !rc; p++) {
                m[0 * pl + p] = mu[3 * p + 0];
                m[1 * pl + p] = mu[3 * p + 1];
                m[2 * pl + p] = ep[3 * p + 2];
                m[3 * pl + p] = ep[3 * p + 1];
                m[4 * pl + p] = ep[3 * p + 0];
                m[5 * pl + p] = mu[3 * p + 2];
            }
        }
    }
    /* Xi files (initial_calc :190-191, final_calc :298-299): the bottom port's for
     * both ends when the targets are the same or the second is a bottom layer */
    const int top_xi = !same && target[1][0] != 'B';
    if (!rc) {
        char name[BUF + 32];
        snprintf(name, sizeof name, "%s_bXi.dat", prefix);
        rc = scalc_xi(name, NA, &xiB);
        if (!rc && top_xi) {
            snprintf(name, sizeof name, "%s_tXi.dat", prefix);
            rc = scalc_xi(name, NA, &xiT);
        }
    }
    const int N = nreal[0] + nreal[1];
    const int both_ways = both[0] == 'Y' || both[0] == 'y';
    smat_scalc_info info = {0, 0, 0, 0};
    if (!rc) {
        S = calloc((size_t)N * N, sizeof(double complex));
        if (!S) rc = smat_fail(SMAT_ENOMEM, "Scalc: out of host memory");
    }
    if (!rc) {
        fprintf(stderr, "Forward calc.: iway = 1%s\n", both_ways ? ", then Backward calc.: iway = -1" : "");
        rc = smat_scalc(L[0], L[1], bc, omega, nl, (const double *)meds, (const double *)xiB, nreal[0],
                        (const double *)(top_xi ? xiT : xiB), nreal[1], both_ways, (double *)S, &info);
    }
    if (!rc) { /* Out_Smat :113-140 */
        char name[BUF + 32];
        snprintf(name, sizeof name, "%s_Smatrix.dat", prefix);
        FILE *f = fopen(name, "w");
        if (!f) rc = smat_fail(SMAT_EINVAL, "open error!: open o-file!");
        else {
            time_t t_f = time(0);
            fprintf(f, "# This file          : ' %s ' on %s", name, ctime(&t_f));
            fprintf(f, "# Exec. file         : ' %s ' (smatranem_gb300, GPU layer transfer)\n", argv[0]);
            fprintf(f, "# Calc. time         : Exec. time = %1.0f s\n", difftime(t_f, t_ini));
            fprintf(f, "# Parameter file     : ' %s ' for prefix, boundary conditions and internal precision\n",
                    argv[1]);
            fprintf(f, "# Omega              : k/k_0 = %.20e\n", omega);
            fprintf(f, "# Boundary conditions: B0 = %d, B1 = %d\n", bc[0], bc[1]);
            fprintf(f, "# Target layers      : Bottom = %s, Top = %s\n", target[0], target[1]);
            fprintf(f, "# Mode numbers       : Bottom = %d, Top = %d\n", nreal[0], nreal[1]);
            fprintf(f, "# Calc. mode         : both ways = %s, 'zgesv' = %s\n", both, solv);
            fprintf(f, "# Smat. residual norm: unitarity = %.16e, transpose = %.16e\n", info.unitarity,
                    info.transpose);
            fprintf(f, "# m n real(S_mn) imag(S_mn) |S_mn|^2 for m,n < %d\n", N);
            for (int c = 0; c < N; c++)
                for (int r = 0; r < N; r++) {
                    const double complex v = S[r + (size_t)N * c];
                    const double a = cabs(v);
                    fprintf(f, "%d %d %.20e %.20e %.20e\n", r, c, creal(v), cimag(v), a * a);
                }
            fclose(f);
        }
    }
    free(meds), free(mu), free(ep), free(xiB), free(xiT), free(S);
    if (rc) {
        fprintf(stderr, "%s\n", smat_last_error());
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}
