/*
 * fpl_oracle.h -- CPU oracle for the phase-linking hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This header and fpl_oracle.c restate, on the
 * CPU and in FP64, the per-pixel loop of FRInGE's evd / phase_link modules
 * (src/evd/evd.cpp:512-788, src/phase_link/phase_link.cpp:479-666) so that
 * the GPU library can be checked against it.  Only the test-suite, the smoke
 * check and the CPU-baseline leg of the benchmark may load it; the product
 * library never links or calls it.
 *
 * Two builds share the same loop source:
 *   - libfpl_oracle.so  ("port"): the eigen/inverse primitives are this
 *     project's own restatement of LAPACK's published algorithms
 *     (zhetrd-style Householder tridiagonalisation, dstebz-style bisection,
 *     dstein-style inverse iteration, zpotrf/zpotri-style Cholesky inverse).
 *   - oracle/_ref/libfpl_ref.so ("reference"): the same loop, but the
 *     primitives are the reference's own unmodified EVWorker
 *     (include/fringe/EigenLapack.hpp:60-251) linked against a LAPACK.  It
 *     can only be built where the reference sources are present.
 *
 * Array layouts follow the reference's in-memory layouts:
 *   stack  : complex64, band-planar [nbands][rows][cols]  (arma cx_fmat
 *            cpxdata(cols*rows, nbands), src/evd/evd.cpp:195)
 *   nmap   : uint32 [rows][cols][nulong]                  (arma Mat<uint>
 *            wts(nulong, pixels), src/evd/evd.cpp:197)
 *   phase  : complex64, band-planar [nbands][rows][cols]
 *   tcorr  : float [rows][cols]
 *   comp   : complex64 [rows][cols]
 * Complex values are stored as interleaved (re, im) pairs.
 */
#ifndef FPL_ORACLE_H
#define FPL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { FPL_ORACLE_MLE = 0, FPL_ORACLE_EVD = 1, FPL_ORACLE_STBAS = 2 };
enum { FPL_ORACLE_SEM_EVD = 0, FPL_ORACLE_SEM_PHASE_LINK = 1 };

typedef struct {
    int rows, cols, nbands;
    int ny, nx;               /* half windows (lines, pixels) */
    int method;               /* FPL_ORACLE_MLE / EVD / STBAS */
    int semantics;            /* FPL_ORACLE_SEM_EVD / SEM_PHASE_LINK */
    int mini_stack_count;     /* reference index = mini_stack_count - 1 */
    int band_width;           /* STBAS only */
    int min_neighbors;        /* phase_link semantics only */
    int row_begin, row_end;   /* output rows computed: [row_begin, row_end) */
    int nthreads;             /* <= 0: OpenMP default */
} fpl_oracle_params;

/* Runs the per-pixel loop over rows [row_begin,row_end).  Output arrays are
 * full-size; only the selected rows are written (zeros for skipped pixels,
 * as the reference's per-block zeroing does, src/evd/evd.cpp:447-454).
 * npix (optional, may be NULL) receives the SHP count of each pixel
 * (0 where the centre bit is clear).  Returns 0, or -1 on bad parameters. */
int fpl_oracle_run(const fpl_oracle_params *p, const float *stack,
                   const uint32_t *nmap, float *phase, float *tcorr,
                   float *comp, int32_t *npix);

/* Primitive under test: one eigenpair by 1-based ascending index of a
 * Hermitian matrix A (column-major, n x n, interleaved complex, upper
 * triangle referenced, destroyed), like EVWorker::eigenWithIndex
 * (include/fringe/EigenLapack.hpp:131-202).  w[0] receives the eigenvalue,
 * z (n complex) the eigenvector when want_vec != 0.  Returns LAPACK-style info. */
int fpl_oracle_eig_index(int n, double *A, int index, int want_vec,
                         double *w, double *z);

/* Primitive under test: Hermitian positive-definite inverse in place, like
 * EVWorker::positiveDefiniteInverse (include/fringe/EigenLapack.hpp:217-251).
 * Returns 0 or the 1-based order of the first non-positive pivot. */
int fpl_oracle_pd_inverse(int n, double *A);

/* ---- SHP neighbourhood map (fpl_nmap_oracle.c) ---------------------------
 * The in-memory core of the nmap module (src/nmap/nmap.cpp:345-473) with
 * the two-sample Kolmogorov-Smirnov (KS2) or Anderson-Darling (AD2) test
 * (nmapOptions::method, src/nmap/nmap.cpp:27-40).  stack as above; mask optional
 * [rows][cols] (0 = excluded); amp_const optional per-band amplitude
 * calibration constants (the "amplitudeConstant" item of each band, <= 0 or
 * NULL meaning 1); nmap [rows][cols][nulong] in the Ulongmask layout; count
 * optional [rows][cols] (set bits, centre included).  Returns 0 or -1. */
typedef struct {
    int rows, cols, nbands;
    int ny, nx;               /* half windows (lines, pixels) */
    double prob;              /* similarity threshold (nmapOptions::prob) */
    int nthreads;             /* <= 0: OpenMP default */
    int method;               /* FPL_NMAP_KS2 or FPL_NMAP_AD2 */
} fpl_nmap_params;

#define FPL_NMAP_KS2 0
#define FPL_NMAP_AD2 1

int fpl_oracle_nmap(const fpl_nmap_params *p, const float *stack, const uint8_t *mask,
                    const double *amp_const, uint32_t *nmap, int32_t *count);

/* The probability of one two-sample test of ascending arrays of length n
 * (a is the reference's first argument, the centre pixel). */
double fpl_oracle_ks2(int n, const float *a, const float *b);
double fpl_oracle_ad2(int n, const float *a, const float *b);

/* Which primitive provider this build uses: "port" or "reference". */
const char *fpl_oracle_kind(void);

#ifdef __cplusplus
}
#endif
#endif
