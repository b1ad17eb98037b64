// nmap.cu -- statistically homogeneous pixels (the nmap bitmask) on the GPU.
//
// Replaces the in-memory core of FRInGE's nmap module
// (src/nmap/nmap.cpp:345-473) and its GPU sketch (src/nmap/nmap_cuda.cu:
// 243-334, one thread per pixel with a bubble sort, not built by the
// reference).  For every pixel the amplitudes of its N dates are compared
// with those of each window neighbour by the two-sample Kolmogorov-Smirnov
// test (src/nmap/KS2sample.hpp:96-144); the neighbour's bit is set in the
// Ulongmask layout (include/fringe/ulongmask.hpp:55-74) when the test's
// probability is at least the threshold.
//
//   k_nmap_sort  (thread per pixel): amplitudes |x_b| / alpha_b exactly as
//                the reference forms them (the float modulus is
//                sqrt(x^2 + y^2) in FP64 rounded to float, the division by
//                the calibration constant in FP64), the validity mask
//                (nonzero, not NaN, optional input mask), and an ascending
//                bitonic sort in registers; sorted amplitudes are written
//                date-planar [N][pixel].
//   k_nmap_fwd<0> (CTA per 32-column x TR-row tile): the sorted amplitudes
//                of the tile and of the window rows below and beside it are
//                staged in shared memory; each thread tests its pixel
//                against the neighbours of the forward half window (the
//                offsets of the reference's loop, src/nmap/nmap.cpp:399-416:
//                rows 0..Ny below, and on its own row the columns right of
//                it), merging the two sorted samples to obtain the KS
//                statistic D (in steps of 1/N; a run of equal values in both
//                samples is one step, as in the reference).  The probability
//                depends on D alone, so the decision is a table lookup
//                prepared on the host with the reference's Kolmogorov
//                series.  The results go to a bit array, one bit per pixel
//                and forward offset.
//   k_nmap_mirror (thread per pixel): the map as the reference sets it
//                (nmap.cpp:447-462): a pixel's forward bits are its own
//                tests, its backward bits those of the neighbour whose
//                forward offset reaches it; the count is their sum.  Each
//                pair is tested once.
//   k_nmap_fwd<1> the same forward tests with the two-sample Anderson-Darling
//                test (src/nmap/AD2unique.hpp:270-347).  The statistic is a
//                sum over the merged walk, (2n m_j - n(j+1))^2 /
//                ((j+1)(2n-j-1)) for the j+1 first values of which m_j come
//                from the first sample, and the p-value decreases with it:
//                the host finds the largest sum S* whose p-value, computed as
//                the reference computes it, passes the threshold.  Each
//                thread sums in FP32 and decides when it is clear of S* by
//                a margin far above its rounding; otherwise it repeats the
//                reference's own FP64 sum, operation for operation, and
//                compares that with S*.  Ties are merged second sample
//                first, so the test is not symmetric: like the reference,
//                each pair is tested with the pixel whose forward half
//                window reaches the other as the first sample.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "fringe_gb300.h"
#include "guard.h"

namespace fpl {
namespace {

constexpr int NM_TC = 32;            // tile columns (one warp per tile row)
constexpr int NM_MAX_TR = 16;        // tile rows at most (512 threads)

struct NmapParams {
    const float2 *stack;             // [nb][rows][cols]
    const uint8_t *mask;             // optional [rows][cols]
    float *sorted;                   // [nb][rows*cols]
    uint8_t *valid;                  // [rows*cols]
    uint32_t *nmap;                  // [rows*cols][nulong]
    uint32_t *fwd;                   // [rows*cols][fw]: forward half-window results
    int32_t *count;                  // optional [rows*cols]
    double alpha[FPL_MAX_BANDS];     // normalised calibration constants
    unsigned long long pass_lo;      // KS2: bit k (k < 64): D = k passes the threshold
    unsigned pass_hi;                // KS2: bit 0: D = 64 passes
    double ad_star;                  // AD2: largest walk sum whose p-value passes
    float ad_lo, ad_hi;              // AD2: FP32 sums below ad_lo pass, above ad_hi fail
    int ad_mode;                     // AD2: 0 compare, 1 every pair passes, 2 none does
    float ad_w[2 * FPL_MAX_BANDS];   // AD2: n^2 / ((j+1)(2n-j-1)), j < 2n - 1
    long long plane;
    int rows, cols, nb, ny, nx, nulong, tr, fw;
    int unit_alpha;                  // all constants 1: no division
};

template <int NPAD>
__global__ void k_nmap_sort(NmapParams P)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P.plane) return;
    float v[NPAD];
    bool ok = P.mask ? P.mask[q] != 0 : true;
#pragma unroll
    for (int b = 0; b < NPAD; ++b) {
        v[b] = INFINITY;
        if (b < P.nb) {
            const float2 x = __ldg(P.stack + b * P.plane + q);
            // float modulus as the reference's std::abs(complex<float>):
            // sqrt(x^2 + y^2) in FP64, rounded to float
            const double m2 = __dadd_rn(__dmul_rn((double)x.x, (double)x.x), __dmul_rn((double)x.y, (double)x.y));
            float a = __double2float_rn(__dsqrt_rn(m2));
            if (!P.unit_alpha) a = __double2float_rn(__ddiv_rn((double)a, P.alpha[b]));   // nmap.cpp:374
            ok = ok && a != 0.f && !isnan(a);
            v[b] = a;
        }
    }
    P.valid[q] = ok ? 1 : 0;
    if (!ok) return;
    // ascending bitonic sort (padding +inf stays at the end)
#pragma unroll
    for (int k = 2; k <= NPAD; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
            for (int i = 0; i < NPAD; ++i) {
                const int l = i ^ j;
                if (l > i) {
                    const float a = v[i], c = v[l];
                    if ((i & k) == 0) {
                        v[i] = fminf(a, c);
                        v[l] = fmaxf(a, c);
                    } else {
                        v[i] = fmaxf(a, c);
                        v[l] = fminf(a, c);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int b = 0; b < NPAD; ++b)
        if (b < P.nb) P.sorted[b * P.plane + q] = v[b];
}

// KS statistic of two ascending samples of length n read from shared
// memory with stride `st`, in units of 1/n: the largest |#b - #a| over the
// checkpoints of the merged walk (the reference checks after every single
// step and after each run of values equal in both samples, and once more
// when a sample is exhausted).
__device__ __forceinline__ int ks_steps(const float *A, const float *B, int st, int n)
{
    int ia = 0, ib = 0, d = 0, dm = 0;
    float va = A[0], vb = B[0];
    for (int it = 0; it < 2 * n; ++it) {
        if (va != vb) {
            const bool lt = va < vb;
            d += lt ? -1 : 1;
            ia += lt ? 1 : 0;
            ib += lt ? 0 : 1;
        } else {
            const float x = va;
            while (ia < n && A[ia * st] == x) { --d; ++ia; }
            while (ib < n && B[ib * st] == x) { ++d; ++ib; }
        }
        if (ia >= n || ib >= n) break;
        va = A[ia * st];
        vb = B[ib * st];
        dm = max(dm, abs(d));
    }
    return max(dm, abs(d));
}

// AD2: the walk sum of the first sample a over the merged order of two
// ascending samples (a value of a goes first only when strictly smaller),
// in FP32: the terms d^2 w_j, d = 2 m_j - (j + 1).
__device__ __forceinline__ float ad_walk_fast(const float *A, const float *B, int st, int n, const float *w)
{
    int ia = 0, ib = 0;
    float va = A[0], vb = B[0], s = 0.f;
    for (int j = 0; j < 2 * n - 1; ++j) {
        const bool ta = ia < n && (ib >= n || va < vb);
        if (ta) {
            ++ia;
            if (ia < n) va = A[ia * st];
        } else {
            ++ib;
            if (ib < n) vb = B[ib * st];
        }
        const int d = 2 * ia - (j + 1);
        s = fmaf((float)(d * d), w[j], s);
    }
    return s;
}

// The same sum as the reference evaluates it (src/nmap/AD2unique.hpp:
// 295-309), operation for operation in FP64: bit-identical to the host's.
__device__ double ad_walk_exact(const float *A, const float *B, int st, int n)
{
    int ia = 0, ib = 0;
    const double N = 2.0 * n, dn = n;
    double m = 0.0, s = 0.0;
    for (int j = 0; j < 2 * n - 1; ++j) {
        const bool ta = ia < n && (ib >= n || A[ia * st] < B[ib * st]);
        if (ta) ++ia; else ++ib;
        m = __dadd_rn(m, ta ? 1.0 : 0.0);
        const double bj = j + 1;
        const double t = __dsub_rn(__dmul_rn(N, m), __dmul_rn(dn, bj));
        s = __dadd_rn(s, __ddiv_rn(__dmul_rn(t, t), __dmul_rn(bj, __dsub_rn(N, bj))));
    }
    return s;
}

template <int AD2>
__global__ void __launch_bounds__(NM_TC * NM_MAX_TR) k_nmap_fwd(NmapParams P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    // the tile and the window rows below and beside it: forward offsets
    // reach rows 0..Ny below and columns -Nx..Nx
    const int HW = NM_TC + 2 * P.nx, HH = P.tr + P.ny, HP = HW * HH;
    // odd stride between dates: lanes whose merge walks sit at different
    // positions spread over the banks
    const int SP = HP | 1;
    float *S = reinterpret_cast<float *>(smem);                       // [nb][SP]
    uint8_t *V = smem + sizeof(float) * (size_t)P.nb * SP;           // [HP]
    __shared__ float W[2 * FPL_MAX_BANDS];
    if (AD2)
        for (int j = threadIdx.x; j < 2 * P.nb - 1; j += blockDim.x) W[j] = P.ad_w[j];
    const int ntc = (P.cols + NM_TC - 1) / NM_TC;
    const int R0 = (blockIdx.x / ntc) * P.tr, C0 = (blockIdx.x % ntc) * NM_TC;
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int e = tid; e < HP; e += nth) {
        const int hr = e / HW, hc = e - hr * HW;
        const int r = R0 + hr, c = C0 - P.nx + hc;
        const bool in = r < P.rows && c >= 0 && c < P.cols;
        V[e] = in ? P.valid[(long long)r * P.cols + c] : 0;
    }
    for (int e = tid; e < P.nb * HP; e += nth) {
        const int b = e / HP, h = e - b * HP;
        const int hr = h / HW, hc = h - hr * HW;
        const int r = R0 + hr, c = C0 - P.nx + hc;
        const bool in = r < P.rows && c >= 0 && c < P.cols;
        S[b * SP + h] = in ? __ldg(P.sorted + b * P.plane + (long long)r * P.cols + c) : 0.f;
    }
    __syncthreads();
    const int tr = tid / NM_TC, tc = tid % NM_TC;
    const int r = R0 + tr, c = C0 + tc;
    if (tr >= P.tr || r >= P.rows || c >= P.cols) return;
    const long long q = (long long)r * P.cols + c;
    const int wx = 2 * P.nx + 1, K = (2 * P.ny + 1) * wx, fc = P.ny * wx + P.nx;
    uint32_t *out = P.fwd + q * P.fw;
    const int hp = tr * HW + (tc + P.nx);
    const bool pv = V[hp] != 0;
    uint32_t word = 0;
    int ii = 0, jj = 0;                               // offset of forward tap g = f - fc
    for (int g = 0; g < K - fc; ++g) {
        if (pv) {
            const int hq = hp + ii * HW + jj;
            bool set = false;
            if (V[hq]) {
                if (g == 0) {
                    set = true;                                  // the centre (nmap.cpp:441-445)
                } else if (!AD2) {
                    const int D = ks_steps(S + hp, S + hq, SP, P.nb);
                    set = (D < 64) ? ((P.pass_lo >> D) & 1ull) != 0 : (P.pass_hi & 1u) != 0;
                } else if (P.ad_mode != 0) {
                    set = P.ad_mode == 1;
                } else {
                    // this pixel is the reference's first sample
                    const float sf = ad_walk_fast(S + hp, S + hq, SP, P.nb, W);
                    if (sf < P.ad_lo) set = true;
                    else if (sf > P.ad_hi) set = false;
                    else set = ad_walk_exact(S + hp, S + hq, SP, P.nb) <= P.ad_star;
                }
            }
            if (set) word |= 1u << (g & 31);
        }
        if ((g & 31) == 31 || g == K - fc - 1) {
            out[g >> 5] = word;
            word = 0;
        }
        if (++jj > P.nx) {
            jj = -P.nx;
            ++ii;
        }
    }
}

// the map and count of every pixel from the forward results
__global__ void __launch_bounds__(256) k_nmap_mirror(NmapParams P)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P.plane) return;
    const int r = int(q / P.cols), c = int(q - (long long)r * P.cols);
    const int wx = 2 * P.nx + 1, K = (2 * P.ny + 1) * wx, fc = P.ny * wx + P.nx;
    uint32_t *out = P.nmap + q * P.nulong;
    const uint32_t *own = P.fwd + q * P.fw;
    int cnt = 0;
    uint32_t word = 0;
    int ii = -P.ny, jj = -P.nx;                       // offset of tap f
    for (int f = 0; f < K; ++f) {
        bool set;
        if (f >= fc) {
            const int g = f - fc;
            set = (__ldg(own + (g >> 5)) >> (g & 31)) & 1u;
        } else {
            // the neighbour's forward test at the mirrored offset
            // (nmap.cpp:459): ii <= 0, so the neighbour is never below
            const int rq = r + ii, cq = c + jj, g = fc - f;
            set = rq >= 0 && cq >= 0 && cq < P.cols &&
                  ((__ldg(P.fwd + ((long long)rq * P.cols + cq) * P.fw + (g >> 5)) >> (g & 31)) & 1u);
        }
        if (set) {
            word |= 1u << (f & 31);
            ++cnt;
        }
        if ((f & 31) == 31 || f == K - 1) {
            out[f >> 5] = word;
            word = 0;
        }
        if (++jj > P.nx) {
            jj = -P.nx;
            ++ii;
        }
    }
    if (P.count) P.count[q] = cnt;
}

// The Kolmogorov distribution as the reference evaluates it
// (src/nmap/KS2sample.hpp:42-78, ROOT's KolmogorovProb series).
double kolmogorov_prob(double z)
{
    const double u = std::fabs(z);
    if (u < 0.2) return 1.0;
    if (u < 0.755) {
        const double v = 1.0 / (u * u);
        return 1.0 - 2.50662827 * (std::exp(-1.2337005501361697 * v) + std::exp(-11.103304951225528 * v) +
                                   std::exp(-30.842513753404244 * v)) / u;
    }
    if (u < 6.8116) {
        double r[4] = {0.0, 0.0, 0.0, 0.0};
        const double v = u * u;
        const int maxj = std::max(1, (int)std::round(3.0 / u));
        for (int j = 0; j < maxj; ++j) r[j] = std::exp(-2.0 * (j + 1) * (j + 1) * v);
        return 2.0 * (r[0] - r[1] + r[2] - r[3]);
    }
    return 0.0;
}

// Decisions for D = 0..n.  The reference accumulates the statistic as a
// double sum of +-1/n steps, which lands within a few units in the last
// place of k/n; a table entry is accepted only when the decision is the
// same over that whole interval (false: the threshold sits on the rounding
// of a table value).
// ---- AD2: the reference's p-value as a function of the walk sum ----------
// Scholz & Stephens (1987), "K-sample Anderson-Darling tests", JASA 82:918:
// the m = 1 column of their table of critical points of the standardised
// statistic (the entries the reference reads, src/nmap/AD2unique.hpp:8-48
// at indices 0, 8, .., 272), with the upper-tail probabilities it lists.
const double kAdCrit[35] = {
    -1.1954, -1.1786, -1.166, -1.1407, -1.1253, -1.0777, -1.0489, -0.9978, -0.9417, -0.8981, -0.8598, -0.7258,
    -0.5966, -0.4572, -0.2966, -0.1009, 0.1571, 0.5357, 1.2255, 1.5262, 1.9633, 2.7314, 3.7825, 4.1241, 4.6044,
    5.409, 6.4954, 6.8279, 7.2755, 8.1885, 9.3061, 9.6132, 10.0989, 10.8825, 11.8537};
const double kAdProb[35] = {
    .00001, .00005, .0001, .0005, .001, .005, .01, .025, .05, .075, .1, .2, .3, .4, .5, .6, .7, .8, .9,
    .925, .95, .975, .99, .9925, .995, .9975, .999, .99925, .9995, .99975, .9999, .999925, .99995, .999975,
    .99999};

// sigma_N of the standardised statistic (Scholz & Stephens eq. 4, k = 2,
// both samples of n; N = 2n < 2000, harmonic sums summed in the
// reference's order, src/nmap/AD2unique.hpp:173-219)
double ad_sigma(int n)
{
    const int N = 2 * n;
    const double kk = 2.0, H = 1.0 / (1.0 * n) + 1.0 / (1.0 * n);
    std::vector<double> inv(N > 1 ? N : 2, 0.0);
    double h = 0.0, g = 0.0;
    for (int i = 1; i < N; ++i) {
        inv[i] = 1.0 / i;
        h += inv[i];
    }
    for (int i = 1; i < N - 1; ++i) {
        const double t = inv[N - i];
        for (int j = i + 1; j < N; ++j) g += t * inv[j];
    }
    const double k2 = kk * kk;
    const double a = (4 * g - 6) * (kk - 1) + (10 - 6 * g) * H;
    const double b = (2 * g - 4) * k2 + 8 * h * kk + (2 * g - 14 * h - 4) * H - 8 * h + 4 * g - 6;
    const double c = (6 * h + 2 * g - 2) * k2 + (4 * h - 4 * g + 6) * kk + (2 * h - 6) * H + 4 * h;
    const double d = (2 * h + 6) * k2 - 4 * h * kk;
    const double dN = (double)N;
    double s2 = 0.0;
    s2 += a * (dN * dN * dN) + b * (dN * dN) + c * N + d;
    s2 /= ((double)(N - 1) * (double)(N - 2) * (double)(N - 3));
    return std::sqrt(s2);
}

// the reference's p-value of the standardised statistic t (linear in
// log((1 - p) / p) between the table's points, extrapolated past its ends)
double ad_pvalue(double t)
{
    int i1 = -1;
    for (int i = 0; i < 35; ++i) {
        i1 = i - 1;
        if (t <= kAdCrit[i]) break;
    }
    int i2 = i1 + 1;
    if (i1 < 0) { i1 = 0; i2 = 1; }
    if (i2 >= 35) { i1 = 33; i2 = 34; }
    const double l1 = std::log((1.0 - kAdProb[i1]) / kAdProb[i1]), l2 = std::log((1.0 - kAdProb[i2]) / kAdProb[i2]);
    const double t1 = kAdCrit[i1], t2 = kAdCrit[i2];
    const double l0 = (l1 - l2) * (t - t2) / (t1 - t2) + l2;
    return std::exp(l0) / (1. + std::exp(l0));
}

// does the walk sum s of a pair of n-date samples pass? (the chain of
// src/nmap/AD2unique.hpp:333-345: both samples' sums are s)
bool ad_pass(double s, int n, double sigma, double prob)
{
    double akn = 0.0;
    akn = akn + s / (n * 1.0);
    akn = akn + s / (n * 1.0);
    akn = akn / (2.0 * n);
    double t = akn - 1;
    t /= sigma;
    return ad_pvalue(t) >= prob;
}

// AD2 decision for this stack depth and threshold: the largest passing sum
// S* (the pass set is every sum up to it); false when the decisions
// within 4096 units in the last place of S* are not all on their side of it
// (the threshold sits on the rounding of the p-value there).
bool ad_table(int n, double prob, NmapParams *P)
{
    const double sigma = ad_sigma(n);
    std::memset(P->ad_w, 0, sizeof(P->ad_w));
    for (int j = 0; j < 2 * n - 1; ++j)
        P->ad_w[j] = (float)((double)n * n / ((double)(j + 1) * (double)(2 * n - j - 1)));
    const double top = 1e300;
    const bool p0 = ad_pass(0.0, n, sigma, prob), p1 = ad_pass(top, n, sigma, prob);
    P->ad_star = 0.0;
    P->ad_lo = P->ad_hi = 0.f;
    if (p0 == p1) {                       // one decision for every sum
        P->ad_mode = p0 ? 1 : 2;
        for (int k = 0; k < 64; ++k)
            if (ad_pass(top * k / 64.0, n, sigma, prob) != p0) return false;
        return true;
    }
    if (!p0) return false;                // the p-value must fall with the sum
    auto bits = [](double x) { uint64_t u; std::memcpy(&u, &x, 8); return u; };
    auto val = [](uint64_t u) { double x; std::memcpy(&x, &u, 8); return x; };
    uint64_t lo = bits(0.0), hi = bits(top);
    while (hi - lo > 1) {
        const uint64_t mid = lo + (hi - lo) / 2;
        if (ad_pass(val(mid), n, sigma, prob)) lo = mid; else hi = mid;
    }
    for (int64_t k = -4096; k <= 4096; ++k) {
        const int64_t u = (int64_t)lo + k;
        if (u < 0) continue;
        if (ad_pass(val((uint64_t)u), n, sigma, prob) != (k <= 0)) return false;
    }
    const double star = val(lo);
    P->ad_star = star;
    P->ad_lo = (float)(star * (1.0 - 1e-4));
    P->ad_hi = (float)(star * (1.0 + 1e-4));
    P->ad_mode = 0;
    return true;
}

bool ks_table(int n, double prob, unsigned long long *lo, unsigned *hi)
{
    *lo = 0;
    *hi = 0;
    const double rn = n, s = 1.0 / rn, scale = std::sqrt(rn * rn / (rn + rn));
    for (int k = 0; k <= n; ++k) {
        double acc = 0.0;
        for (int t = 0; t < k; ++t) acc += s;
        const double cand[4] = {acc, k * s, acc * (1.0 - 64 * 1.2e-16), acc * (1.0 + 64 * 1.2e-16)};
        int pass = -1;
        for (double x : cand) {
            const int p = kolmogorov_prob(x * scale) >= prob ? 1 : 0;
            if (pass < 0) pass = p;
            else if (p != pass) return false;
        }
        if (pass) {
            if (k < 64) *lo |= 1ull << k;
            else *hi |= 1u;
        }
    }
    return true;
}

// shared memory of a k_nmap_fwd tile of tr rows: the tile and Ny rows below
size_t nm_tile_smem(int nb, int ny, int nx, int tr)
{
    const int HW = NM_TC + 2 * nx;
    const size_t per_row = (size_t)HW * (sizeof(float) * nb + 1);
    return per_row * (tr + ny) + sizeof(float) * nb;             // + the odd-stride pad per date
}

// tile rows of k_nmap_fwd: the height whose resident warps per SM (CTAs
// that fit in shared memory times warps per CTA) is largest -- the merge
// walks are latency-bound -- preferring taller tiles, which share their
// apron among more pixels.  0 when not even one row fits.
template <typename K>
int nm_tile_rows(K kern, int nb, int ny, int nx, size_t *smem)
{
    int best = 0, best_warps = 0;
    for (int tr = 1; tr <= NM_MAX_TR; ++tr) {
        const size_t sm = nm_tile_smem(nb, ny, nx, tr);
        if (sm > 227 * 1024) break;
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) break;
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NM_TC * tr, sm) != cudaSuccess) break;
        if (per_sm * tr >= best_warps && per_sm > 0) {
            best_warps = per_sm * tr;
            best = tr;
        }
    }
    if (best > 0) *smem = nm_tile_smem(nb, ny, nx, best);
    return best;
}

}  // namespace
}  // namespace fpl

extern "C" int fpl_nmap(fpl_ctx *ctx, const fpl_nmap_job *job)
{
    return fpl_guard([&]() -> int {
        using namespace fpl;
        if (!ctx || !job || !job->stack || !job->nmap) return FPL_ERR_NULL;
        if (job->rows <= 0 || job->cols <= 0 || job->nbands <= 0 || job->half_window_x < 0 ||
            job->half_window_y < 0)
            return FPL_ERR_OPTIONS;
        if (job->memory != FPL_MEM_HOST && job->memory != FPL_MEM_DEVICE) return FPL_ERR_OPTIONS;
        if (!(job->prob >= 0.0) || job->prob > 1.0) return FPL_ERR_OPTIONS;
        if (job->nbands > FPL_MAX_BANDS) return FPL_ERR_UNSUPPORTED;
        const int wx = 2 * job->half_window_x + 1, K = (2 * job->half_window_y + 1) * wx;
        const int nul = (K + 31) / 32;
        if (nul > FPL_MAX_NULONG) return FPL_ERR_UNSUPPORTED;
        NmapParams P;
        std::memset(&P, 0, sizeof(P));
        P.rows = job->rows;
        P.cols = job->cols;
        P.nb = job->nbands;
        P.ny = job->half_window_y;
        P.nx = job->half_window_x;
        P.nulong = nul;
        P.plane = (long long)job->rows * job->cols;
        // calibration constants normalised to the first band (nmap.cpp:204-230)
        double a[FPL_MAX_BANDS];
        for (int b = 0; b < P.nb; ++b) {
            const double cst = job->amp_const ? job->amp_const[b] : 1.0;
            a[b] = cst > 0.0 ? cst : 1.0;
        }
        const double a0 = a[0];
        for (int b = 0; b < P.nb; ++b) a[b] /= a0;
        a[0] = 1.0;
        P.unit_alpha = 1;
        for (int b = 0; b < P.nb; ++b) {
            P.alpha[b] = a[b];
            if (a[b] != 1.0) P.unit_alpha = 0;
        }
        if (job->method != FPL_NMAP_KS2 && job->method != FPL_NMAP_AD2) return FPL_ERR_OPTIONS;
        const bool ad2 = job->method == FPL_NMAP_AD2;
        if (!ad2 && !ks_table(P.nb, job->prob, &P.pass_lo, &P.pass_hi)) {
            ctx->last_error = "the threshold lies within rounding of a Kolmogorov table value for this stack depth";
            return FPL_ERR_OPTIONS;
        }
        if (ad2 && !ad_table(P.nb, job->prob, &P)) {
            ctx->last_error = "the threshold lies within rounding of the Anderson-Darling p-value for this stack depth";
            return FPL_ERR_OPTIONS;
        }
        if (cudaSetDevice(ctx->device) != cudaSuccess) return FPL_ERR_CUDA;
        auto kern = ad2 ? k_nmap_fwd<1> : k_nmap_fwd<0>;
        size_t smem = 0;
        P.tr = nm_tile_rows(kern, P.nb, P.ny, P.nx, &smem);
        if (P.tr <= 0) return FPL_ERR_UNSUPPORTED;
        cudaStream_t st = ctx->stream;
        const size_t b_stack = (size_t)P.plane * P.nb * 8, b_nmap = (size_t)P.plane * nul * 4;
        const size_t b_sorted = ((size_t)P.plane * P.nb * 4 + 255) & ~size_t(255);   // keeps every region 256-aligned
        // scratch: sorted amplitudes | validity | forward results | (host jobs)
        // mask, stack, nmap, count
        P.fw = ((K - (P.ny * wx + P.nx)) + 31) / 32;
        const size_t b_fwd = ((size_t)P.plane * P.fw * 4 + 255) & ~size_t(255);
        size_t need = b_sorted + ((P.plane + 255) & ~255ll) + b_fwd;
        if (job->memory == FPL_MEM_HOST)
            need += ((b_stack + 255) & ~size_t(255)) + ((b_nmap + 255) & ~size_t(255)) +
                    (((size_t)P.plane * 4 + 255) & ~size_t(255)) + (((size_t)P.plane + 255) & ~size_t(255));
        if (ctx->cap_nm < need) {
            if (ctx->d_nm) cudaFree(ctx->d_nm);
            ctx->d_nm = nullptr;
            ctx->cap_nm = 0;
            if (cudaMalloc(&ctx->d_nm, need) != cudaSuccess) return FPL_ERR_NOMEM;
            ctx->cap_nm = need;
        }
        char *base = static_cast<char *>(ctx->d_nm);
        P.sorted = reinterpret_cast<float *>(base);
        base += b_sorted;
        P.valid = reinterpret_cast<uint8_t *>(base);
        base += (P.plane + 255) & ~255ll;
        P.fwd = reinterpret_cast<uint32_t *>(base);
        base += b_fwd;
        auto fail = [&](cudaError_t e, const char *what) {
            ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
            return FPL_ERR_CUDA;
        };
        cudaError_t e;
        if (job->memory == FPL_MEM_HOST) {
            void *d_stack = base;
            base += (b_stack + 255) & ~size_t(255);
            P.nmap = reinterpret_cast<uint32_t *>(base);
            base += (b_nmap + 255) & ~size_t(255);
            P.count = job->count ? reinterpret_cast<int32_t *>(base) : nullptr;
            base += ((size_t)P.plane * 4 + 255) & ~size_t(255);
            uint8_t *d_mask = job->mask ? reinterpret_cast<uint8_t *>(base) : nullptr;
            if ((e = cudaMemcpyAsync(d_stack, job->stack, b_stack, cudaMemcpyHostToDevice, st)) != cudaSuccess)
                return fail(e, "copy stack");
            if (d_mask && (e = cudaMemcpyAsync(d_mask, job->mask, (size_t)P.plane, cudaMemcpyHostToDevice, st)) !=
                              cudaSuccess)
                return fail(e, "copy mask");
            P.stack = static_cast<const float2 *>(d_stack);
            P.mask = d_mask;
        } else {
            P.stack = static_cast<const float2 *>(job->stack);
            P.mask = job->mask;
            P.nmap = job->nmap;
            P.count = job->count;
        }
        const unsigned sblocks = (unsigned)((P.plane + 127) / 128);
        if (P.nb <= 16) k_nmap_sort<16><<<sblocks, 128, 0, st>>>(P);
        else if (P.nb <= 32) k_nmap_sort<32><<<sblocks, 128, 0, st>>>(P);
        else k_nmap_sort<64><<<sblocks, 128, 0, st>>>(P);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "k_nmap_sort");
        if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
            return fail(e, "k_nmap_fwd attributes");
        const long long ntiles = (long long)((P.cols + NM_TC - 1) / NM_TC) * ((P.rows + P.tr - 1) / P.tr);
        kern<<<(unsigned)ntiles, NM_TC * P.tr, smem, st>>>(P);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "k_nmap_fwd");
        k_nmap_mirror<<<(unsigned)((P.plane + 255) / 256), 256, 0, st>>>(P);
        if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "k_nmap_mirror");
        if (job->memory == FPL_MEM_HOST) {
            if ((e = cudaMemcpyAsync(job->nmap, P.nmap, b_nmap, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
                return fail(e, "copy nmap");
            if (job->count &&
                (e = cudaMemcpyAsync(job->count, P.count, (size_t)P.plane * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
                return fail(e, "copy count");
        }
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e, "fpl_nmap");
        return FPL_OK;
    });
}
