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
//   k_nmap_ks    (CTA per 32-column x TR-row tile): the sorted amplitudes of
//                the tile and its window apron are staged in shared memory;
//                each thread walks its pixel's taps and, for each valid
//                neighbour, merges the two sorted samples to obtain the KS
//                statistic D (in steps of 1/N; a run of equal values in both
//                samples is one step, as in the reference).  The probability
//                depends on D alone, so the decision is a table lookup
//                prepared on the host with the reference's Kolmogorov
//                series.  The test is symmetric, so testing every neighbour
//                of every pixel gives the reference's half-window-and-mirror
//                map exactly.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"
#include "fringe_gb300.h"

namespace fpl {
namespace {

constexpr int NM_TC = 32;            // tile columns (one warp per tile row)

struct NmapParams {
    const float2 *stack;             // [nb][rows][cols]
    const uint8_t *mask;             // optional [rows][cols]
    float *sorted;                   // [nb][rows*cols]
    uint8_t *valid;                  // [rows*cols]
    uint32_t *nmap;                  // [rows*cols][nulong]
    int32_t *count;                  // optional [rows*cols]
    double alpha[FPL_MAX_BANDS];     // normalised calibration constants
    unsigned long long pass_lo;      // bit k (k < 64): D = k passes the threshold
    unsigned pass_hi;                // bit 0: D = 64 passes
    long long plane;
    int rows, cols, nb, ny, nx, nulong, tr;
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

__global__ void __launch_bounds__(256) k_nmap_ks(NmapParams P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int HW = NM_TC + 2 * P.nx, HH = P.tr + 2 * P.ny, HP = HW * HH;
    // odd stride between dates: lanes whose merge walks sit at different
    // positions spread over the banks
    const int SP = HP | 1;
    float *S = reinterpret_cast<float *>(smem);                       // [nb][SP]
    uint8_t *V = smem + sizeof(float) * (size_t)P.nb * SP;           // [HP]
    const int ntc = (P.cols + NM_TC - 1) / NM_TC;
    const int R0 = (blockIdx.x / ntc) * P.tr, C0 = (blockIdx.x % ntc) * NM_TC;
    const int tid = threadIdx.x, nth = blockDim.x;
    // tile + apron: sorted amplitudes and validity
    for (int e = tid; e < HP; e += nth) {
        const int hr = e / HW, hc = e - hr * HW;
        const int r = R0 - P.ny + hr, c = C0 - P.nx + hc;
        const bool in = r >= 0 && r < P.rows && c >= 0 && c < P.cols;
        V[e] = in ? P.valid[(long long)r * P.cols + c] : 0;
    }
    for (int e = tid; e < P.nb * HP; e += nth) {
        const int b = e / HP, h = e - b * HP;
        const int hr = h / HW, hc = h - hr * HW;
        const int r = R0 - P.ny + hr, c = C0 - P.nx + hc;
        const bool in = r >= 0 && r < P.rows && c >= 0 && c < P.cols;
        S[b * SP + h] = in ? __ldg(P.sorted + b * P.plane + (long long)r * P.cols + c) : 0.f;
    }
    __syncthreads();
    const int tr = tid / NM_TC, tc = tid % NM_TC;
    const int r = R0 + tr, c = C0 + tc;
    if (tr >= P.tr || r >= P.rows || c >= P.cols) return;
    const long long q = (long long)r * P.cols + c;
    const int wx = 2 * P.nx + 1, K = (2 * P.ny + 1) * wx;
    uint32_t *out = P.nmap + q * P.nulong;
    const int hp = (tr + P.ny) * HW + (tc + P.nx);
    const bool pv = V[hp] != 0;
    int cnt = 0;
    uint32_t word = 0;
    for (int f = 0; f < K; ++f) {
        if (pv) {
            const int ii = f / wx - P.ny, jj = f % wx - P.nx;
            const int hq = hp + ii * HW + jj;
            bool set = false;
            if (V[hq]) {
                if (hq == hp) {
                    set = true;                                  // the centre (nmap.cpp:441-445)
                } else {
                    const int D = ks_steps(S + hp, S + hq, SP, P.nb);
                    set = (D < 64) ? ((P.pass_lo >> D) & 1ull) != 0 : (P.pass_hi & 1u) != 0;
                }
            }
            if (set) {
                word |= 1u << (f & 31);
                ++cnt;
            }
        }
        if ((f & 31) == 31 || f == K - 1) {
            out[f >> 5] = word;
            word = 0;
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

int nm_tile_rows(int nb, int ny, int nx, size_t *smem)
{
    const int HW = NM_TC + 2 * nx;
    const size_t per_row = (size_t)HW * (sizeof(float) * nb + 1);
    const size_t budget = 200 * 1024;
    int tr = 8;
    while (tr > 1 && per_row * (tr + 2 * ny) + sizeof(float) * nb > budget) --tr;
    *smem = per_row * (tr + 2 * ny) + sizeof(float) * nb;        // + the odd-stride pad per date
    return *smem <= 227 * 1024 ? tr : 0;
}

}  // namespace
}  // namespace fpl

extern "C" int fpl_nmap(fpl_ctx *ctx, const fpl_nmap_job *job)
{
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
    if (!ks_table(P.nb, job->prob, &P.pass_lo, &P.pass_hi)) {
        ctx->last_error = "the threshold lies within rounding of a Kolmogorov table value for this stack depth";
        return FPL_ERR_OPTIONS;
    }
    size_t smem = 0;
    P.tr = nm_tile_rows(P.nb, P.ny, P.nx, &smem);
    if (P.tr <= 0) return FPL_ERR_UNSUPPORTED;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return FPL_ERR_CUDA;
    cudaStream_t st = ctx->stream;
    const size_t b_stack = (size_t)P.plane * P.nb * 8, b_nmap = (size_t)P.plane * nul * 4;
    const size_t b_sorted = ((size_t)P.plane * P.nb * 4 + 255) & ~size_t(255);   // keeps every region 256-aligned
    // scratch: sorted amplitudes | validity | (host jobs) mask, stack, nmap, count
    size_t need = b_sorted + ((P.plane + 255) & ~255ll);
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
    if ((e = cudaFuncSetAttribute(k_nmap_ks, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024)) != cudaSuccess)
        return fail(e, "k_nmap_ks attributes");
    const long long ntiles = (long long)((P.cols + NM_TC - 1) / NM_TC) * ((P.rows + P.tr - 1) / P.tr);
    k_nmap_ks<<<(unsigned)ntiles, NM_TC * P.tr, smem, st>>>(P);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "k_nmap_ks");
    if (job->memory == FPL_MEM_HOST) {
        if ((e = cudaMemcpyAsync(job->nmap, P.nmap, b_nmap, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
            return fail(e, "copy nmap");
        if (job->count &&
            (e = cudaMemcpyAsync(job->count, P.count, (size_t)P.plane * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
            return fail(e, "copy count");
    }
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e, "fpl_nmap");
    return FPL_OK;
}
