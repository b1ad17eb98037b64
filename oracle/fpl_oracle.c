/*
 * fpl_oracle.c -- CPU oracle (FP64) for the phase-linking hot path.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by the test-suite, the smoke check and
 * the CPU-baseline leg of the benchmark, never by the product library.
 *
 * The per-pixel loop restates src/evd/evd.cpp:512-788 (evd semantics) and
 * src/phase_link/phase_link.cpp:479-666 (phase_link semantics) with plain
 * arrays in place of Armadillo cubes and without GDAL.  Arithmetic follows
 * the reference: products of complex64 samples are formed in FP32 and
 * accumulated in FP64, everything after the gather is FP64.
 *
 * Built without FPL_BACKEND_REF ("port"), the eigen-pair and inverse
 * primitives are restatements of LAPACK's published algorithms, which the
 * reference calls through EVWorker (include/fringe/EigenLapack.hpp:131-251):
 *   zheevr(JOBZ, RANGE='I', UPLO='U', IL=IU=index) -> for a single index
 *       LAPACK reduces to tridiagonal form (zhetrd), finds the eigenvalue by
 *       bisection (dstebz), the vector by inverse iteration (zstein) and
 *       back-transforms it (zunmtr);
 *   zpotrf('U') + zpotri('U')     -> Cholesky A = U^H U and inv(U) inv(U)^H.
 * LAPACK itself is a third-party dependency of the reference (its CMake asks
 * for any LAPACK, CMakeLists.txt:25, no version pinned).
 *
 * Built with FPL_BACKEND_REF, the primitives are the reference's own EVWorker
 * (see ref_backend.cpp) and the result is the reference's numerics.
 */
#include "fpl_oracle.h"

#include <complex.h>
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex zc;

/* ------------------------------------------------------------------------ */
/* Ulongmask bit layout: include/fringe/ulongmask.hpp:81-94.                 */
/* offset (ii,jj) in [-Ny,Ny]x[-Nx,Nx] -> flat=(ii+Ny)(2Nx+1)+jj+Nx,         */
/* word flat/32, bit flat%32, LSB first.                                     */
/* ------------------------------------------------------------------------ */
static inline int getbit(const uint32_t *arr, int ny, int nx, int ii, int jj)
{
    (void)ny;
    int flat = (ii + ny) * (2 * nx + 1) + jj + nx;
    return (int)((arr[flat / 32] >> (flat % 32)) & 1u);
}

#ifndef FPL_BACKEND_REF
/* ======================================================================== */
/* "port" primitives                                                         */
/* ======================================================================== */

typedef struct {
    int n;
    zc *tau;      /* n   Householder scalars            */
    zc *p;        /* n   work vector                    */
    double *d;    /* n   tridiagonal diagonal           */
    double *e;    /* n   tridiagonal off-diagonal       */
    double *y;    /* n   eigenvector of T               */
    double *lu;   /* 5n  LU factors of T - lambda I     */
    int *piv;     /* n                                  */
    zc *u;        /* n*n Cholesky / inverse workspace   */
} port_ws;

static void *ws_create(int n)
{
    port_ws *w = (port_ws *)calloc(1, sizeof(port_ws));
    w->n = n;
    w->tau = (zc *)calloc((size_t)n, sizeof(zc));
    w->p = (zc *)calloc((size_t)n, sizeof(zc));
    w->d = (double *)calloc((size_t)n, sizeof(double));
    w->e = (double *)calloc((size_t)n, sizeof(double));
    w->y = (double *)calloc((size_t)n, sizeof(double));
    w->lu = (double *)calloc((size_t)5 * n, sizeof(double));
    w->piv = (int *)calloc((size_t)n, sizeof(int));
    w->u = (zc *)calloc((size_t)n * n, sizeof(zc));
    return w;
}

static void ws_destroy(void *v)
{
    port_ws *w = (port_ws *)v;
    if (!w) return;
    free(w->tau); free(w->p); free(w->d); free(w->e); free(w->y);
    free(w->lu); free(w->piv); free(w->u); free(w);
}

/* Householder reduction of a Hermitian matrix to real symmetric tridiagonal
 * form, Q^H A Q = T, Q = H(0) H(1) ... H(n-2), H(k) = I - tau_k v_k v_k^H.
 * Restates LAPACK zhetd2 (lower variant) and zlarfg.  a is full column-major
 * storage; both triangles are read and kept Hermitian.  On return the
 * reflector v_k occupies a[k+1.., k] with the leading 1 implied. */
static void port_tridiag(int n, zc *a, double *d, double *e, zc *tau, zc *p)
{
    for (int k = 0; k < n - 1; ++k) {
        const int m = n - k - 1;
        zc *x = &a[(k + 1) + (size_t)k * n];
        zc alpha = x[0];
        double scale = 0.0, ssq = 1.0;          /* scaled 2-norm of x[1..m) */
        for (int i = 1; i < m; ++i) {
            double c[2] = {creal(x[i]), cimag(x[i])};
            for (int t = 0; t < 2; ++t) {
                double v = fabs(c[t]);
                if (v != 0.0) {
                    if (scale < v) { ssq = 1.0 + ssq * (scale / v) * (scale / v); scale = v; }
                    else ssq += (v / scale) * (v / scale);
                }
            }
        }
        double xnorm = scale * sqrt(ssq);
        double ar = creal(alpha), ai = cimag(alpha);
        zc t;
        if (xnorm == 0.0 && ai == 0.0) {
            t = 0.0;
            e[k] = ar;
        } else {
            double nrm = sqrt(ar * ar + ai * ai + xnorm * xnorm);
            double beta = (ar >= 0.0) ? -nrm : nrm;
            t = (beta - ar) / beta - I * (ai / beta);
            zc s = 1.0 / (alpha - beta);
            for (int i = 1; i < m; ++i) x[i] *= s;
            e[k] = beta;
        }
        tau[k] = t;
        x[0] = 1.0;
        if (t != 0.0) {
            zc *a22 = &a[(k + 1) + (size_t)(k + 1) * n];
            /* p = t * A22 * v */
            for (int i = 0; i < m; ++i) {
                zc s = 0.0;
                for (int j = 0; j < m; ++j) s += a22[i + (size_t)j * n] * x[j];
                p[i] = t * s;
            }
            /* w = p - 1/2 t (p^H v) v */
            zc pv = 0.0;
            for (int i = 0; i < m; ++i) pv += conj(p[i]) * x[i];
            zc K = -0.5 * t * pv;
            for (int i = 0; i < m; ++i) p[i] += K * x[i];
            /* A22 -= v w^H + w v^H */
            for (int j = 0; j < m; ++j)
                for (int i = 0; i < m; ++i)
                    a22[i + (size_t)j * n] -= x[i] * conj(p[j]) + p[i] * conj(x[j]);
        }
    }
    for (int k = 0; k < n; ++k) d[k] = creal(a[k + (size_t)k * n]);
}

/* Number of eigenvalues of T (d, e) below sigma: Sturm count via the LDL^T
 * recurrence, as LAPACK dstebz / dlaebz use it. */
static int sturm_count(int n, const double *d, const double *e, double sigma,
                       double pivmin)
{
    int cnt = 0;
    double q = d[0] - sigma;
    if (fabs(q) <= pivmin) q = -pivmin;
    if (q < 0.0) cnt++;
    for (int i = 1; i < n; ++i) {
        q = d[i] - sigma - e[i - 1] * e[i - 1] / q;
        if (fabs(q) <= pivmin) q = -pivmin;
        if (q < 0.0) cnt++;
    }
    return cnt;
}

/* index-th (1-based ascending) eigenvalue of T by bisection (dstebz). */
static double port_bisect(int n, const double *d, const double *e, int index,
                          double *tnorm_out)
{
    double gl = d[0], gu = d[0], emax2 = 0.0;
    for (int i = 0; i < n; ++i) {
        double r = 0.0;
        if (i > 0) r += fabs(e[i - 1]);
        if (i < n - 1) { r += fabs(e[i]); if (e[i] * e[i] > emax2) emax2 = e[i] * e[i]; }
        if (d[i] - r < gl) gl = d[i] - r;
        if (d[i] + r > gu) gu = d[i] + r;
    }
    double pivmin = DBL_MIN * (emax2 > 1.0 ? emax2 : 1.0);
    double tnorm = fmax(fabs(gl), fabs(gu));
    double fudge = 2.1 * DBL_EPSILON * tnorm * n + 2.0 * pivmin;
    double lo = gl - fudge, hi = gu + fudge;
    for (int it = 0; it < 256; ++it) {
        double mid = 0.5 * (lo + hi);
        double tol = 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + pivmin;
        if (hi - lo <= tol || mid <= lo || mid >= hi) break;
        if (sturm_count(n, d, e, mid, pivmin) >= index) hi = mid; else lo = mid;
    }
    if (tnorm_out) *tnorm_out = tnorm;
    return 0.5 * (lo + hi);
}

/* Eigenvector of T for eigenvalue lam by inverse iteration (dstein): LU with
 * partial pivoting of T - lam I (dlagtf), triangular solves (dlagts). */
static void port_inverse_iteration(int n, const double *d, const double *e,
                                   double lam, double tnorm, double *y,
                                   double *lu, int *piv)
{
    double *dg = lu, *u1 = lu + n, *u2 = lu + 2 * n, *l = lu + 3 * n;
    double eps = DBL_EPSILON * (tnorm > 0.0 ? tnorm : 1.0);
    for (int i = 0; i < n; ++i) {
        dg[i] = d[i] - lam;
        u1[i] = (i < n - 1) ? e[i] : 0.0;
        u2[i] = 0.0;
        l[i] = 0.0;
        piv[i] = 0;
    }
    /* factor: rows i and i+1, sub-diagonal e[i] */
    for (int i = 0; i < n - 1; ++i) {
        double sub = e[i];
        if (fabs(dg[i]) >= fabs(sub)) {
            if (dg[i] == 0.0) dg[i] = eps;
            l[i] = sub / dg[i];
            dg[i + 1] -= l[i] * u1[i];
            piv[i] = 0;
        } else {
            /* swap rows i and i+1 */
            double mult = dg[i] / sub;
            double old_u1 = u1[i];
            dg[i] = sub;
            u1[i] = dg[i + 1];
            u2[i] = (i < n - 2) ? u1[i + 1] : 0.0;
            dg[i + 1] = old_u1 - mult * u1[i];
            if (i < n - 2) u1[i + 1] = -mult * u2[i];
            l[i] = mult;
            piv[i] = 1;
        }
    }
    if (dg[n - 1] == 0.0) dg[n - 1] = eps;

    /* deterministic start vector */
    unsigned s = 12345u;
    for (int i = 0; i < n; ++i) {
        s = s * 1103515245u + 12345u;
        y[i] = ((double)((s >> 8) & 0xFFFF) / 65535.0) - 0.5 + 1.0;
    }
    for (int it = 0; it < 4; ++it) {
        /* forward: apply L^{-1} with the row interchanges */
        for (int i = 0; i < n - 1; ++i) {
            if (piv[i]) { double t = y[i]; y[i] = y[i + 1]; y[i + 1] = t - l[i] * y[i]; }
            else y[i + 1] -= l[i] * y[i];
        }
        /* back substitution with U (diag dg, super u1, super-2 u2) */
        for (int i = n - 1; i >= 0; --i) {
            double t = y[i];
            if (i + 1 < n) t -= u1[i] * y[i + 1];
            if (i + 2 < n) t -= u2[i] * y[i + 2];
            y[i] = t / dg[i];
        }
        double mx = 0.0;
        for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(y[i]));
        if (mx == 0.0 || !isfinite(mx)) { for (int i = 0; i < n; ++i) y[i] = 1.0; continue; }
        for (int i = 0; i < n; ++i) y[i] /= mx;
    }
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) nrm += y[i] * y[i];
    nrm = sqrt(nrm);
    for (int i = 0; i < n; ++i) y[i] /= nrm;
}

/* zheevr(RANGE='I', IL=IU=index) semantics: eigenvalue and (optionally)
 * eigenvector of the Hermitian matrix whose upper triangle is in A. */
static int ws_eig(void *vw, zc *A, int index, int want_vec, double *w, zc *z)
{
    port_ws *ws = (port_ws *)vw;
    const int n = ws->n;
    if (index < 1 || index > n) return -9;
    /* complete the lower triangle from the upper (UPLO='U') */
    for (int j = 0; j < n; ++j) {
        A[j + (size_t)j * n] = creal(A[j + (size_t)j * n]);
        for (int i = j + 1; i < n; ++i) A[i + (size_t)j * n] = conj(A[j + (size_t)i * n]);
    }
    for (int i = 0; i < n * n; ++i)
        if (!isfinite(creal(A[i])) || !isfinite(cimag(A[i]))) return n + 1;
    if (n == 1) {
        w[0] = creal(A[0]);
        if (want_vec) z[0] = 1.0;
        return 0;
    }
    port_tridiag(n, A, ws->d, ws->e, ws->tau, ws->p);
    double tnorm;
    double lam = port_bisect(n, ws->d, ws->e, index, &tnorm);
    w[0] = lam;
    if (!want_vec) return 0;
    port_inverse_iteration(n, ws->d, ws->e, lam, tnorm, ws->y, ws->lu, ws->piv);
    for (int i = 0; i < n; ++i) z[i] = ws->y[i];
    /* z = H(0) H(1) ... H(n-2) y */
    for (int k = n - 2; k >= 0; --k) {
        zc t = ws->tau[k];
        if (t == 0.0) continue;
        const zc *v = &A[(k + 1) + (size_t)k * n];   /* v[0] == 1 */
        zc s = 0.0;
        for (int i = 0; i < n - k - 1; ++i) s += conj(v[i]) * z[k + 1 + i];
        s *= t;
        for (int i = 0; i < n - k - 1; ++i) z[k + 1 + i] -= s * v[i];
    }
    return 0;
}

/* zpotrf('U') + zpotri('U') + Hermitian fill, as
 * EVWorker::positiveDefiniteInverse (include/fringe/EigenLapack.hpp:217-251). */
static int ws_pdinv(void *vw, zc *A)
{
    port_ws *ws = (port_ws *)vw;
    const int n = ws->n;
    zc *U = A;   /* factor in place, upper triangle */
    for (int j = 0; j < n; ++j) {
        double ajj = creal(U[j + (size_t)j * n]);
        for (int k = 0; k < j; ++k) {
            zc ukj = U[k + (size_t)j * n];
            ajj -= creal(ukj) * creal(ukj) + cimag(ukj) * cimag(ukj);
        }
        if (ajj <= 0.0 || isnan(ajj)) return j + 1;
        double ujj = sqrt(ajj);
        U[j + (size_t)j * n] = ujj;
        for (int i = j + 1; i < n; ++i) {
            zc s = U[j + (size_t)i * n];
            for (int k = 0; k < j; ++k) s -= conj(U[k + (size_t)j * n]) * U[k + (size_t)i * n];
            U[j + (size_t)i * n] = s / ujj;
        }
    }
    /* inv(U) into ws->u (upper) */
    zc *V = ws->u;
    memset(V, 0, sizeof(zc) * (size_t)n * n);
    for (int j = 0; j < n; ++j) {
        V[j + (size_t)j * n] = 1.0 / U[j + (size_t)j * n];
        for (int i = j - 1; i >= 0; --i) {
            zc s = 0.0;
            for (int k = i + 1; k <= j; ++k) s += U[i + (size_t)k * n] * V[k + (size_t)j * n];
            V[i + (size_t)j * n] = -s / U[i + (size_t)i * n];
        }
    }
    /* inv(A) = V V^H, upper triangle */
    for (int j = 0; j < n; ++j)
        for (int i = 0; i <= j; ++i) {
            zc s = 0.0;
            for (int k = j; k < n; ++k) s += V[i + (size_t)k * n] * conj(V[j + (size_t)k * n]);
            A[i + (size_t)j * n] = s;
        }
    /* Hermitian fill of the lower triangle (EigenLapack.hpp:240-248) */
    for (int ii = 0; ii < n; ++ii)
        for (int jj = ii + 1; jj < n; ++jj) A[ii * n + jj] = conj(A[jj * n + ii]);
    return 0;
}

const char *fpl_oracle_kind(void) { return "port"; }

#else
/* ======================================================================== */
/* "reference" primitives: the reference's EVWorker (ref_backend.cpp)        */
/* ======================================================================== */
void *fpl_ref_ws_create(int n);
void fpl_ref_ws_destroy(void *w);
int fpl_ref_ws_eig(void *w, double *A, int index, int want_vec, double *val,
                   double *vec);
int fpl_ref_ws_pdinv(void *w, double *A);

static void *ws_create(int n) { return fpl_ref_ws_create(n); }
static void ws_destroy(void *w) { fpl_ref_ws_destroy(w); }
static int ws_eig(void *w, zc *A, int index, int want_vec, double *val, zc *z)
{
    return fpl_ref_ws_eig(w, (double *)A, index, want_vec, val, (double *)z);
}
static int ws_pdinv(void *w, zc *A) { return fpl_ref_ws_pdinv(w, (double *)A); }
const char *fpl_oracle_kind(void) { return "reference"; }
#endif

/* ------------------------------------------------------------------------ */
/* exported primitives                                                        */
/* ------------------------------------------------------------------------ */
int fpl_oracle_eig_index(int n, double *A, int index, int want_vec, double *w,
                         double *z)
{
    void *ws = ws_create(n);
    int info = ws_eig(ws, (zc *)A, index, want_vec, w, (zc *)z);
    ws_destroy(ws);
    return info;
}

int fpl_oracle_pd_inverse(int n, double *A)
{
    void *ws = ws_create(n);
    int info = ws_pdinv(ws, (zc *)A);
    ws_destroy(ws);
    return info;
}

/* ------------------------------------------------------------------------ */
/* per-pixel loop                                                             */
/* ------------------------------------------------------------------------ */
int fpl_oracle_run(const fpl_oracle_params *p, const float *stack,
                   const uint32_t *nmap, float *phase, float *tcorr,
                   float *comp, int32_t *npix_out)
{
    if (!p || !stack || !nmap || !phase || !tcorr || !comp) return -1;
    const int rows = p->rows, cols = p->cols, nb = p->nbands;
    const int Ny = p->ny, Nx = p->nx;
    if (rows <= 0 || cols <= 0 || nb <= 0 || Ny < 0 || Nx < 0) return -1;
    const int mini = p->mini_stack_count;
    if (mini < 1 || mini > nb) return -1;
    const int isstbas = (p->method == FPL_ORACLE_STBAS);
    const int ismle = (p->method == FPL_ORACLE_MLE);
    const int plink = (p->semantics == FPL_ORACLE_SEM_PHASE_LINK);
    const int BW = p->band_width;
    if (isstbas && (BW <= 0 || BW >= nb - 1)) return -1;   /* evd.cpp:74-91 */
    const int r0 = p->row_begin < 0 ? 0 : p->row_begin;
    const int r1 = p->row_end > rows ? rows : p->row_end;
    const int numAround = (2 * Ny + 1) * (2 * Nx + 1);
    const int nulong = (numAround + 31) / 32;
    const size_t plane = (size_t)rows * cols;
    /* evd.cpp:566 hard-codes 2; phase_link.cpp:524 honours minNeighbors */
    const int minNeigh = plink ? p->min_neighbors : 2;

#ifdef _OPENMP
    if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#pragma omp parallel
#endif
    {
        zc *Numer = (zc *)malloc(sizeof(zc) * nb * nb);
        zc *Covar = (zc *)malloc(sizeof(zc) * nb * nb);
        zc *Amp1 = (zc *)malloc(sizeof(zc) * nb * nb);
        zc *Amp2 = (zc *)malloc(sizeof(zc) * nb * nb);
        zc *vec = (zc *)malloc(sizeof(zc) * nb);
        double *P = (double *)malloc(sizeof(double) * nb);
        float *xs = (float *)malloc(sizeof(float) * 2 * nb);
        void *ws = ws_create(nb);
        double eigval = 0.0;

#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (long pp = (long)r0 * cols; pp < (long)r1 * cols; ++pp) {
            /* zero outputs (the reference zeroes its block buffers) */
            for (int b = 0; b < nb; ++b) {
                phase[2 * (b * plane + pp)] = 0.f;
                phase[2 * (b * plane + pp) + 1] = 0.f;
            }
            tcorr[pp] = 0.f;
            comp[2 * pp] = 0.f;
            comp[2 * pp + 1] = 0.f;
            if (npix_out) npix_out[pp] = 0;

            const uint32_t *cen = nmap + (size_t)pp * nulong;
            if (getbit(cen, Ny, Nx, 0, 0) == 0) continue;          /* evd.cpp:517 */

            const int cenii = (int)(pp / cols), cenjj = (int)(pp % cols);
            const int xmin = cenjj - Nx > 0 ? cenjj - Nx : 0;     /* evd.cpp:530-534 */
            const int xmax = cenjj + Nx < cols - 1 ? cenjj + Nx : cols - 1;
            const int ymin = cenii - Ny > 0 ? cenii - Ny : 0;
            const int ymax = cenii + Ny < rows - 1 ? cenii + Ny : rows - 1;

            memset(Numer, 0, sizeof(zc) * nb * nb);
            memset(P, 0, sizeof(double) * nb);
            int npix = 0;
            /* gather + accumulation, evd.cpp:539-564.  Amp1(ti,tj) and
             * Amp2(ti,tj) only ever accumulate |x_ti|^2 and |x_tj|^2 in the
             * same order for every partner, so one per-date sum P[t] holds
             * the identical FP64 value. */
            for (int ii = ymin; ii <= ymax; ++ii)
                for (int jj = xmin; jj <= xmax; ++jj) {
                    if (!getbit(cen, Ny, Nx, ii - cenii, jj - cenjj)) continue;
                    npix++;
                    const size_t q = (size_t)ii * cols + jj;
                    for (int t = 0; t < nb; ++t) {
                        xs[2 * t] = stack[2 * (t * plane + q)];
                        xs[2 * t + 1] = stack[2 * (t * plane + q) + 1];
                        float ab = hypotf(xs[2 * t], xs[2 * t + 1]);   /* std::abs(complex<float>) */
                        P[t] += (double)ab * (double)ab;                /* std::pow(.,2) in double */
                    }
                    for (int ti = 0; ti < nb; ++ti) {
                        const float a = xs[2 * ti], b = xs[2 * ti + 1];
                        for (int tj = ti + 1; tj < nb; ++tj) {
                            const float c = xs[2 * tj], d = xs[2 * tj + 1];
                            /* complex<float> x_ti * conj(x_tj), in FP32 */
                            const float re = a * c + b * d;
                            const float im = b * c - a * d;
                            Numer[ti + tj * nb] += (double)re + I * (double)im;
                        }
                    }
                }
            if (npix_out) npix_out[pp] = npix;
            if (npix < minNeigh) continue;                          /* evd.cpp:566 */

            /* coherence, evd.cpp:569-582 */
            for (int ti = 0; ti < nb; ++ti) {
                for (int tj = ti + 1; tj < nb; ++tj) {
                    zc res = Numer[ti + tj * nb] / sqrt(P[ti] * P[tj]);
                    Covar[ti + tj * nb] = res;
                    Covar[tj + ti * nb] = conj(res);
                }
                Covar[ti + ti * nb] = 1.0;
            }

            int solved = 0;
            if (!plink) {
                if (ismle) {
                    /* |Covar| into Amp1, evd.cpp:587-596 */
                    for (int ti = 0; ti < nb; ++ti) {
                        for (int tj = ti + 1; tj < nb; ++tj) {
                            double coh = cabs(Covar[ti + tj * nb]);
                            Amp1[ti + tj * nb] = coh;
                            Amp1[tj + ti * nb] = coh;
                        }
                        Amp1[ti + ti * nb] = 1.0;
                    }
                    memcpy(Amp2, Covar, sizeof(zc) * nb * nb);      /* evd.cpp:600-620 */
                    int st = ws_eig(ws, Amp2, 1, 0, &eigval, vec);
                    if (st != 0) { tcorr[pp] = -1.f; continue; }
                    if (eigval < 1.0e-6) { tcorr[pp] = -2.f; continue; }
                    memcpy(Amp2, Amp1, sizeof(zc) * nb * nb);       /* evd.cpp:623-644 */
                    st = ws_eig(ws, Amp2, 1, 0, &eigval, vec);
                    if (st != 0) { tcorr[pp] = -3.f; continue; }
                    if (eigval < 1.0e-6) { tcorr[pp] = -4.f; continue; }
                    memcpy(Amp2, Amp1, sizeof(zc) * nb * nb);       /* evd.cpp:652-664 */
                    st = ws_pdinv(ws, Amp2);
                    if (st != 0) { tcorr[pp] = -5.f; continue; }
                    for (int i = 0; i < nb * nb; ++i) Amp2[i] *= Covar[i];   /* evd.cpp:667 */
                    st = ws_eig(ws, Amp2, 1, 1, &eigval, vec);      /* evd.cpp:670-686 */
                    if (st != 0) { tcorr[pp] = -6.f; continue; }
                    if (eigval < 1.0e-6) { tcorr[pp] = -7.f; continue; }
                    solved = 1;
                } else {
                    if (isstbas) {                                  /* evd.cpp:695-706 */
                        for (int ti = 0; ti < nb; ++ti)
                            for (int tj = ti + BW + 1; tj < nb; ++tj) {
                                Covar[tj + ti * nb] = 0.0;
                                Covar[ti + tj * nb] = 0.0;
                            }
                    }
                    memcpy(Amp1, Covar, sizeof(zc) * nb * nb);      /* evd.cpp:710-730 */
                    int st = ws_eig(ws, Amp1, nb, 1, &eigval, vec);
                    if (st != 0) { tcorr[pp] = -6.f; continue; }
                    if (eigval < 1.0e-6) { tcorr[pp] = -7.f; continue; }
                    solved = 1;
                }
            } else {
                /* phase_link.cpp:540-618 */
                memcpy(Amp1, Covar, sizeof(zc) * nb * nb);
                int st = ws_eig(ws, Amp1, 1, 0, &eigval, vec);
                if (st != 0) { tcorr[pp] = -1.f; continue; }
                for (int ti = 0; ti < nb; ++ti) {
                    for (int tj = ti + 1; tj < nb; ++tj) {
                        double coh = cabs(Covar[ti + tj * nb]);
                        Amp1[ti + tj * nb] = coh;
                        Amp1[tj + ti * nb] = coh;
                    }
                    Amp1[ti + ti * nb] = 1.0;
                }
                int run_evd = 0;
                memcpy(Amp2, Amp1, sizeof(zc) * nb * nb);
                if (ws_pdinv(ws, Amp2) != 0) run_evd = 1;
                if (!run_evd) {
                    for (int i = 0; i < nb * nb; ++i) Amp2[i] *= Covar[i];
                    if (ws_eig(ws, Amp2, 1, 1, &eigval, vec) != 0) run_evd = 1;
                }
                if (run_evd) {
                    memcpy(Amp1, Covar, sizeof(zc) * nb * nb);
                    if (ws_eig(ws, Amp1, nb, 1, &eigval, vec) != 0) { tcorr[pp] = -6.f; continue; }
                }
                solved = 1;
            }
            if (!solved) continue;

            /* phase referencing, evd.cpp:738-749 */
            const double ph0 = carg(vec[mini - 1]);
            for (int b = 0; b < nb; ++b) {
                double res = carg(vec[b]) - ph0;
                phase[2 * (b * plane + pp)] = (float)cos(res);
                phase[2 * (b * plane + pp) + 1] = (float)sin(res);
            }
            phase[2 * ((mini - 1) * plane + pp)] = 1.f;
            phase[2 * ((mini - 1) * plane + pp) + 1] = 0.f;

            /* compressed SLC, evd.cpp:752-762 */
            {
                double sr = 0.0, si = 0.0;
                for (int b = mini - 1; b < nb; ++b) {
                    const float a = stack[2 * (b * plane + pp)], bb = stack[2 * (b * plane + pp) + 1];
                    const float c = phase[2 * (b * plane + pp)], d = phase[2 * (b * plane + pp) + 1];
                    const float re = a * c + bb * d;          /* complex<float> x * conj(ph) */
                    const float im = bb * c - a * d;
                    sr += re;
                    si += im;
                }
                const double den = 1.0 * (nb - mini + 1);
                comp[2 * pp] = (float)(sr / den);
                comp[2 * pp + 1] = (float)(si / den);
            }

            /* temporal coherence, evd.cpp:768-786.  For STBAS the reference's
             * upper limit ti+BW+1 can pass nbands and read outside the matrix;
             * the pairs that exist (tj < nbands) are used here. */
            {
                double sr = 0.0, si = 0.0;
                int counter = 0;
                for (int ti = 0; ti < nb; ++ti) {
                    int ulim = isstbas ? (ti + BW + 1) : nb;
                    if (ulim > nb) ulim = nb;
                    const float argi = atan2f(phase[2 * (ti * plane + pp) + 1], phase[2 * (ti * plane + pp)]);
                    for (int tj = ti + 1; tj < ulim; ++tj) {
                        const float argj = atan2f(phase[2 * (tj * plane + pp) + 1], phase[2 * (tj * plane + pp)]);
                        const double ang = carg(Covar[ti + tj * nb]) - (double)argi + (double)argj;
                        sr += cos(ang);
                        si += sin(ang);
                        counter++;
                    }
                }
                /* 0/0 for a single date, as in the reference */
                tcorr[pp] = (float)(sqrt(sr * sr + si * si) / (counter * 1.0));
            }
        }
        ws_destroy(ws);
        free(Numer); free(Covar); free(Amp1); free(Amp2); free(vec); free(P); free(xs);
    }
    return 0;
}
