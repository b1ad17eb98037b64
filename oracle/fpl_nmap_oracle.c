/*
 * fpl_nmap_oracle.c -- CPU oracle for the SHP neighbourhood map (nmap).
 *
 * TEST INFRASTRUCTURE ONLY.  Restates, on the CPU, the in-memory core of
 * FRInGE's nmap module (src/nmap/nmap.cpp:345-473): per-band amplitudes
 * |x| / alpha_b with a validity mask, ascending sort of each pixel's
 * amplitudes, the two-sample Kolmogorov-Smirnov test of the centre pixel
 * against each window neighbour (src/nmap/KS2sample.hpp:96-144, the
 * KolmogorovTest algorithm of the ROOT library, with the Kolmogorov
 * distribution series of KolmogorovProb, :42-78), and the Ulongmask bit
 * layout (include/fringe/ulongmask.hpp:55-74).  The reference tests each
 * unordered pair once over half a window and mirrors the bit; the test is
 * symmetric, so testing every neighbour of every pixel gives the same map.
 *
 * Built into libfpl_oracle.so ("port").  With -DFPL_BACKEND_REF the test
 * itself is the reference's own KS2sample::test (ref_backend.cpp).
 */
#include "fpl_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#ifdef FPL_BACKEND_REF
double fpl_ref_ks2(int n, const float *a, const float *b);
#define KS_TEST(n, a, b) fpl_ref_ks2((n), (a), (b))
#else
/* Kolmogorov distribution Q(z) = 2 sum_j (-1)^(j-1) exp(-2 j^2 z^2), with
 * the small-z form sqrt(2 pi)/z sum exp(-(2j-1)^2 pi^2 / (8 z^2)) (the
 * series and cut points of ROOT's KolmogorovProb). */
static double ks_prob(double z)
{
    const double u = fabs(z);
    if (u < 0.2) return 1.0;
    if (u < 0.755) {
        const double v = 1.0 / (u * u);
        return 1.0 - 2.50662827 * (exp(-1.2337005501361697 * v) + exp(-11.103304951225528 * v) +
                                   exp(-30.842513753404244 * v)) / u;
    }
    if (u < 6.8116) {
        double r[4] = {0.0, 0.0, 0.0, 0.0};
        const double v = u * u;
        int maxj = (int)round(3.0 / u);
        if (maxj < 1) maxj = 1;
        for (int j = 0; j < maxj; ++j) r[j] = exp(-2.0 * (j + 1) * (j + 1) * v);
        return 2.0 * (r[0] - r[1] + r[2] - r[3]);
    }
    return 0.0;
}

/* two equal-length ascending samples: walk the merged order, the empirical
 * distributions differ by d steps of 1/n; a run of equal values from both
 * samples is one step.  Returns Q(D sqrt(n n / (n + n))). */
static double ks_test(int n, const float *a, const float *b)
{
    const double rn = n, s = 1.0 / rn;
    int ia = 0, ib = 0;
    double d = 0.0, dmax = 0.0;
    for (int i = 0; i < 2 * n; ++i) {
        if (a[ia] < b[ib]) {
            d -= s;
            ++ia;
        } else if (a[ia] > b[ib]) {
            d += s;
            ++ib;
        } else {
            const float x = a[ia];
            while (ia < n && a[ia] == x) { d -= s; ++ia; }
            while (ib < n && b[ib] == x) { d += s; ++ib; }
        }
        if (ia >= n || ib >= n) break;
        if (dmax < fabs(d)) dmax = fabs(d);
    }
    if (dmax < fabs(d)) dmax = fabs(d);
    return ks_prob(dmax * sqrt(rn * rn / (rn + rn)));
}
#define KS_TEST(n, a, b) ks_test((n), (a), (b))
#endif

static int cmp_float(const void *x, const void *y)
{
    const float a = *(const float *)x, b = *(const float *)y;
    return (a > b) - (a < b);
}

double fpl_oracle_ks2(int n, const float *a, const float *b) { return KS_TEST(n, a, b); }

int fpl_oracle_nmap(const fpl_nmap_params *p, const float *stack, const uint8_t *mask,
                    const double *amp_const, uint32_t *nmap, int32_t *count)
{
    if (!p || !stack || !nmap || p->rows <= 0 || p->cols <= 0 || p->nbands <= 0 || p->ny < 0 || p->nx < 0)
        return -1;
    const int rows = p->rows, cols = p->cols, n = p->nbands;
    const int wx = 2 * p->nx + 1, K = (2 * p->ny + 1) * wx, nul = (K + 31) / 32;
    const long long P = (long long)rows * cols;
    /* calibration constants normalised to the first band; <= 0 means 1
     * (src/nmap/nmap.cpp:204-230) */
    double *alpha = (double *)malloc(sizeof(double) * n);
    for (int b = 0; b < n; ++b) {
        const double c = amp_const ? amp_const[b] : 1.0;
        alpha[b] = c > 0.0 ? c : 1.0;
    }
    const double a0 = alpha[0];
    for (int b = 0; b < n; ++b) alpha[b] /= a0;
    alpha[0] = 1.0;
    /* [pixel][band]; one spare row: the reference's tie loop reads one
     * element past a sample before testing the index */
    float *amp = (float *)malloc(sizeof(float) * ((size_t)P + 1) * n);
    uint8_t *valid = (uint8_t *)malloc((size_t)P);
    if (p->nthreads > 0) omp_set_num_threads(p->nthreads);
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < P; ++q) {
        int ok = mask ? mask[q] != 0 : 1;
        for (int b = 0; b < n; ++b) {
            const float complex x = stack[2 * (b * P + q)] + I * stack[2 * (b * P + q) + 1];
            const float val = (float)(cabsf(x) / alpha[b]);      /* nmap.cpp:373-376 */
            ok = ok && val != 0.f && !isnan(val);
            amp[q * n + b] = val;
        }
        valid[q] = (uint8_t)ok;
        if (ok) qsort(amp + q * n, n, sizeof(float), cmp_float);
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (long long q = 0; q < P; ++q) {
        uint32_t *w = nmap + q * nul;
        memset(w, 0, sizeof(uint32_t) * nul);
        int cnt = 0;
        if (valid[q]) {
            const int r = (int)(q / cols), c = (int)(q % cols);
            for (int ii = -p->ny; ii <= p->ny; ++ii) {
                for (int jj = -p->nx; jj <= p->nx; ++jj) {
                    const int rr = r + ii, cc = c + jj;
                    if (rr < 0 || rr >= rows || cc < 0 || cc >= cols) continue;
                    const long long o = (long long)rr * cols + cc;
                    if (!valid[o]) continue;
                    int set = (o == q);
                    if (!set) set = KS_TEST(n, amp + q * n, amp + o * n) >= p->prob;
                    if (set) {
                        const int f = (ii + p->ny) * wx + (jj + p->nx);
                        w[f >> 5] |= 1u << (f & 31);
                        ++cnt;
                    }
                }
            }
        }
        if (count) count[q] = cnt;
    }
    free(alpha);
    free(amp);
    free(valid);
    return 0;
}
