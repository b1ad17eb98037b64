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
 * layout (include/fringe/ulongmask.hpp:55-74).  The second method is the
 * two-sample Anderson-Darling test (src/nmap/AD2unique.hpp:270-347).  The
 * reference tests each unordered pair once, over half a window, with the
 * earlier pixel of its loop (src/nmap/nmap.cpp:399-416: row offsets 0..Ny,
 * column offsets 0..Nx on the centre row) as the first sample, and mirrors
 * the bit.  The KS test is symmetric; the AD test is not when the samples
 * share values (ties are merged second sample first), so every pair is
 * tested here in the reference's order.
 *
 * Built into libfpl_oracle.so ("port").  With -DFPL_BACKEND_REF the tests
 * themselves are the reference's own KS2sample::test and AD2unique::test
 * (ref_backend.cpp).
 */
#include "fpl_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#ifdef FPL_BACKEND_REF
double fpl_ref_ks2(int n, const float *a, const float *b);
double fpl_ref_ad2(int n, const float *a, const float *b);
#define KS_TEST(n, a, b) fpl_ref_ks2((n), (a), (b))
#define AD_TEST(n, a, b) fpl_ref_ad2((n), (a), (b))
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

/* ---- two-sample Anderson-Darling test --------------------------------------
 * Scholz & Stephens (1987), "K-sample Anderson-Darling tests", JASA 82:918,
 * for k = 2 samples of equal length n, in the form of src/nmap/
 * AD2unique.hpp: the statistic A2akN without the ties adjustment, its
 * standardisation by the exact variance sigma_N (Scholz & Stephens eq. 4
 * with the harmonic sums h and g), and the p-value interpolated linearly in
 * log((1 - p) / p) between the m = 1 column of the paper's table of
 * critical points (the reference reads entries 0, 8, .., 272 of its ts[]). */
static const double ad_crit[35] = {
    -1.1954, -1.1786, -1.166, -1.1407, -1.1253, -1.0777, -1.0489, -0.9978, -0.9417, -0.8981, -0.8598, -0.7258,
    -0.5966, -0.4572, -0.2966, -0.1009, 0.1571, 0.5357, 1.2255, 1.5262, 1.9633, 2.7314, 3.7825, 4.1241, 4.6044,
    5.409, 6.4954, 6.8279, 7.2755, 8.1885, 9.3061, 9.6132, 10.0989, 10.8825, 11.8537};
static const double ad_prob[35] = {
    .00001, .00005, .0001, .0005, .001, .005, .01, .025, .05, .075, .1, .2, .3, .4, .5, .6, .7, .8, .9,
    .925, .95, .975, .99, .9925, .995, .9975, .999, .99925, .9995, .99975, .9999, .999925, .99995, .999975,
    .99999};

/* sigma_N of the standardised statistic for two samples of n each (N = 2n
 * < 2000: the harmonic sums are summed, not approximated) */
static double ad_sigma(int n)
{
    const int N = 2 * n;
    const double kk = 2.0, H = 1.0 / (1.0 * n) + 1.0 / (1.0 * n);
    double h = 0.0, g = 0.0;
    double *inv = (double *)malloc(sizeof(double) * (size_t)(N > 1 ? N : 2));
    for (int i = 1; i < N; ++i) {
        inv[i] = 1.0 / i;
        h += inv[i];
    }
    for (int i = 1; i < N - 1; ++i) {
        const double t = inv[N - i];
        for (int j = i + 1; j < N; ++j) g += t * inv[j];
    }
    free(inv);
    const double k2 = kk * kk;
    const double a = (4 * g - 6) * (kk - 1) + (10 - 6 * g) * H;
    const double b = (2 * g - 4) * k2 + 8 * h * kk + (2 * g - 14 * h - 4) * H - 8 * h + 4 * g - 6;
    const double c = (6 * h + 2 * g - 2) * k2 + (4 * h - 4 * g + 6) * kk + (2 * h - 6) * H + 4 * h;
    const double d = (2 * h + 6) * k2 - 4 * h * kk;
    const double dN = (double)N;
    double s2 = 0.0;
    s2 += a * (dN * dN * dN) + b * (dN * dN) + c * N + d;
    s2 /= ((double)(N - 1) * (double)(N - 2) * (double)(N - 3));
    return sqrt(s2);
}

/* p-value of the standardised statistic t */
static double ad_pvalue(double t)
{
    int i1 = -1;
    for (int i = 0; i < 35; ++i) {
        i1 = i - 1;
        if (t <= ad_crit[i]) break;
    }
    int i2 = i1 + 1;
    if (i1 < 0) { i1 = 0; i2 = 1; }
    if (i2 >= 35) { i1 = 33; i2 = 34; }
    const double l1 = log((1.0 - ad_prob[i1]) / ad_prob[i1]), l2 = log((1.0 - ad_prob[i2]) / ad_prob[i2]);
    const double t1 = ad_crit[i1], t2 = ad_crit[i2];
    const double l0 = (l1 - l2) * (t - t2) / (t1 - t2) + l2;
    return exp(l0) / (1. + exp(l0));
}

/* the statistic's sum over the merged walk for one sample: after step j
 * (j + 1 values taken, m of them from this sample) the term
 * (2n m - n (j + 1))^2 / ((j + 1)(2n - j - 1)), for j < 2n - 1 */
static double ad_walk_sum(int n, const unsigned char *from_a, int want_a)
{
    const double N = 2.0 * n;
    double m = 0.0, s = 0.0;
    for (int j = 0; j < 2 * n; ++j) {
        m += (from_a[j] != 0) == (want_a != 0) ? 1.0 : 0.0;
        const double bj = j + 1;
        if (j < 2 * n - 1) {
            const double t = N * m - n * bj;
            s = s + t * t / (bj * (N - bj));
        }
    }
    return s;
}

static double ad_test(int n, const float *a, const float *b, double sigma)
{
    /* merged order of the two ascending samples: a value of a goes first
     * only when strictly smaller (ties: b first) */
    unsigned char from_a[2 * n];
    int ia = 0, ib = 0, k = 0;
    while (ia < n && ib < n) {
        if (a[ia] < b[ib]) { from_a[k++] = 1; ++ia; }
        else { from_a[k++] = 0; ++ib; }
    }
    while (ib < n) { from_a[k++] = 0; ++ib; }
    while (ia < n) { from_a[k++] = 1; ++ia; }
    const double sa = ad_walk_sum(n, from_a, 1), sb = ad_walk_sum(n, from_a, 0);
    double akn = 0.0;
    akn = akn + sa / (n * 1.0);
    akn = akn + sb / (n * 1.0);
    akn = akn / (2.0 * n);
    double t = akn - 1;
    t /= sigma;
    return ad_pvalue(t);
}
#define AD_TEST(n, a, b) ad_test((n), (a), (b), ad_sig)
#endif

double fpl_oracle_ad2(int n, const float *a, const float *b)
{
#ifndef FPL_BACKEND_REF
    const double ad_sig = ad_sigma(n);
#endif
    return AD_TEST(n, a, b);
}

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
#ifndef FPL_BACKEND_REF
    const double ad_sig = (p->method == FPL_NMAP_AD2) ? ad_sigma(n) : 0.0;
#endif
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
                    if (!set) {
                        /* the reference's first sample: the pixel whose loop
                         * reaches the other one (later row, or same row and
                         * later column) */
                        const int fwd = ii > 0 || (ii == 0 && jj > 0);
                        const float *s0 = fwd ? amp + q * n : amp + o * n, *s1 = fwd ? amp + o * n : amp + q * n;
                        set = (p->method == FPL_NMAP_AD2 ? AD_TEST(n, s0, s1) : KS_TEST(n, s0, s1)) >= p->prob;
                    }
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
