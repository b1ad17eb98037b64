// gram_tc.cu -- coherence matrices on the 5th-generation tensor cores.
//
// Mixed-precision form of the SHP gather + Gamma accumulation
// (src/evd/evd.cpp:539-582).  For one pixel, the N dates of its S SHP
// samples form Y = [Re x; Im x] (64 rows x S, dates padded to 32).  Each
// sample is split into bf16 hi + lo parts and the CTA stages the operand
//     A = [Y_hi ; Y_lo]          (128 rows x S, bf16, K-major)
// in shared memory.  One thread issues tcgen05.mma (M = 128, N = 64, K = 16
// per instruction) with B = Y_hi (the first 64 rows of A), accumulating
//     D = A Y_hi^T = [Y_hi Y_hi^T ; Y_lo Y_hi^T]      (128 x 64, FP32, TMEM)
// over the samples.  Then Y Y^T ~ HH + LH + LH^T (the lo*lo term, ~2^-16
// relative, is dropped), from which
//     Re Gamma_ij = S_ij + S_{32+i,32+j},  Im Gamma_ij = S_{32+i,j} - S_{i,32+j}.
// The four warps read D back with tcgen05.ld (one 32-lane quadrant each),
// stage it in shared memory, normalise Gamma to coherence and store the
// packed upper triangle for the eigen kernel (k_solve).
//
// Operand layout (no swizzle, K-major): core matrices of 8 rows x 16 bytes,
// contiguous; K-adjacent core matrices 128 B apart (LBO), 8-row groups
// KC*16 B apart (SBO).  Every wait on the tensor core is bounded; on timeout
// the CTA records an error flag, skips its remaining pixels and still frees
// its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "pixel.cuh"

namespace fpl {
namespace {

constexpr int TC_THREADS = 128;
constexpr int TC_KC = 128;                        // samples per MMA chunk
constexpr int TC_ROWS = 128;                      // [Re hi; Im hi; Re lo; Im lo] x 32 dates
constexpr int TC_SBO = TC_KC * 16;                // bytes between 8-row groups
constexpr int TC_A_BYTES = TC_ROWS * TC_KC * 2;   // 32 KiB
constexpr int TC_LDD = 65;                        // D staging row stride (floats)
constexpr int TC_D_BYTES = TC_ROWS * TC_LDD * 4;
constexpr int TC_MAXK = 1024;                     // window taps (nulong <= 32)
constexpr int TC_TMEM_COLS = 64;                  // the N = 64 accumulator
// D is staged in the operand buffer, which is free once the MMAs complete
constexpr size_t TC_OFF_D = 0;
constexpr size_t TC_AD_BYTES = (TC_A_BYTES > TC_D_BYTES ? TC_A_BYTES : TC_D_BYTES);
constexpr size_t TC_OFF_SHP = (TC_AD_BYTES + 127) & ~size_t(127);
constexpr size_t TC_OFF_MISC = TC_OFF_SHP + TC_MAXK * 4;
constexpr size_t TC_SMEM = TC_OFF_MISC + 256;
constexpr unsigned ERR_TC_TIMEOUT = 2u;
constexpr long long TC_SPIN_LIMIT = 1ll << 26;    // ~ seconds of polling

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t make_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor, kind::f16: FP32 accumulate, bf16 A and B, both
// K-major, N = 64, M = 128
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void tc_commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_addr(mbar)) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(mbar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *mbar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok) : "r"(smem_addr(mbar)), "r"(parity) : "memory");
    return ok != 0;
}

// 16 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r)
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// byte offset of A(row m, sample k) in the no-swizzle K-major layout
__device__ __forceinline__ uint32_t a_offset(int m, int k)
{
    return (uint32_t)((m >> 3) * TC_SBO + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    const __nv_bfloat16 ha = __float2bfloat16_rn(a), hb = __float2bfloat16_rn(b);
    return (uint32_t)__bfloat16_as_ushort(ha) | ((uint32_t)__bfloat16_as_ushort(hb) << 16);
}
__device__ __forceinline__ float bf16_lo(float x)
{
    return x - __bfloat162float(__float2bfloat16_rn(x));
}

__global__ void __launch_bounds__(TC_THREADS) k_gram_tc(KParams P)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *A = smem;
    float *D = reinterpret_cast<float *>(smem + TC_OFF_D);
    int *shp = reinterpret_cast<int *>(smem + TC_OFF_SHP);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + TC_OFF_MISC);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + TC_OFF_MISC + 8);
    int *wcount = reinterpret_cast<int *>(smem + TC_OFF_MISC + 16);      // 4 warps
    float *rs = reinterpret_cast<float *>(smem + TC_OFF_MISC + 32);      // 1/sqrt(P_i), 32
    int *flag = reinterpret_cast<int *>(smem + TC_OFF_MISC + 160);       // bad / abort

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(tmem_slot)), "r"(TC_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        flag[1] = 0;
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tbase = *tmem_slot;
    const uint32_t a_base = smem_addr(A);
    uint32_t phase = 0;

    const int n = P.nb;
    const int cols = P.cols, rows = P.rows;
    const long long plane = P.plane;
    const bool plink = (P.semantics == SEM_PL);
    const int min_neigh = plink ? P.min_neigh : 2;
    const int npk = n * (n + 1) / 2;
    const unsigned lt = (1u << lane) - 1u;

    for (long long q = blockIdx.x; q < P.npix; q += gridDim.x) {
        const long long pp = P.pix_begin + q;
        const long long loc = pp - P.cbase;
        const uint32_t *cen = P.nmap + pp * P.nulong;
        const int cr = int(pp / cols), cc = int(pp % cols);
        const int cflat = P.ny * P.wx + P.nx;
        if (!((__ldg(cen + (cflat >> 5)) >> (cflat & 31)) & 1u)) {   // evd.cpp:517
            if (tid == 0) P.cinfo[loc] = CI_CENTRE;
            continue;
        }
        // ---- SHP list in tap order (block-wide ballot compaction) ----
        int count = 0;
        for (int f0 = 0; f0 < P.K; f0 += TC_THREADS) {
            const int f = f0 + tid;
            bool set = false;
            int qi = 0;
            if (f < P.K) {
                const int r = cr + f / P.wx - P.ny, c = cc + f % P.wx - P.nx;
                if (r >= 0 && r < rows && c >= 0 && c < cols) {
                    set = (__ldg(cen + (f >> 5)) >> (f & 31)) & 1u;
                    qi = r * cols + c;
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, set);
            if (lane == 0) wcount[warp] = __popc(m);
            __syncthreads();
            int base = count;
            for (int w = 0; w < warp; ++w) base += wcount[w];
            if (set) shp[base + __popc(m & lt)] = qi;
            count += wcount[0] + wcount[1] + wcount[2] + wcount[3];
            __syncthreads();
        }
        const int npix = count;
        if (npix < min_neigh) {                               // evd.cpp:566
            if (tid == 0) P.cinfo[loc] = CI_FEW;
            continue;
        }
        // ---- operand staging and MMAs, TC_KC samples at a time ----
        bool timed_out = false;
        for (int c0 = 0; c0 < npix; c0 += TC_KC) {
            const int len = min(TC_KC, npix - c0);
            const int kpad = (len + 15) & ~15;
            const int ncc = kpad >> 3;                         // 8-sample column chunks
            // task = (date d, 8-sample chunk ck): consecutive threads take
            // consecutive dates, so a warp's 16-byte stores fill whole
            // 128-byte core-matrix rows (no bank conflicts)
#pragma unroll 2
            for (int t = tid; t < 32 * ncc; t += TC_THREADS) {
                const int d = t & 31, ck = t >> 5;
                float re[8], im[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int s = ck * 8 + e;
                    float2 x = make_float2(0.f, 0.f);
                    if (d < n && s < len) x = __ldg(P.stack + d * plane + shp[c0 + s]);
                    re[e] = x.x;
                    im[e] = x.y;
                }
                uint4 rh, ih, rl, il;
                rh.x = pack_bf16(re[0], re[1]); rh.y = pack_bf16(re[2], re[3]);
                rh.z = pack_bf16(re[4], re[5]); rh.w = pack_bf16(re[6], re[7]);
                ih.x = pack_bf16(im[0], im[1]); ih.y = pack_bf16(im[2], im[3]);
                ih.z = pack_bf16(im[4], im[5]); ih.w = pack_bf16(im[6], im[7]);
                rl.x = pack_bf16(bf16_lo(re[0]), bf16_lo(re[1])); rl.y = pack_bf16(bf16_lo(re[2]), bf16_lo(re[3]));
                rl.z = pack_bf16(bf16_lo(re[4]), bf16_lo(re[5])); rl.w = pack_bf16(bf16_lo(re[6]), bf16_lo(re[7]));
                il.x = pack_bf16(bf16_lo(im[0]), bf16_lo(im[1])); il.y = pack_bf16(bf16_lo(im[2]), bf16_lo(im[3]));
                il.z = pack_bf16(bf16_lo(im[4]), bf16_lo(im[5])); il.w = pack_bf16(bf16_lo(im[6]), bf16_lo(im[7]));
                const int k = ck * 8;
                *reinterpret_cast<uint4 *>(A + a_offset(d, k)) = rh;
                *reinterpret_cast<uint4 *>(A + a_offset(32 + d, k)) = ih;
                *reinterpret_cast<uint4 *>(A + a_offset(64 + d, k)) = rl;
                *reinterpret_cast<uint4 *>(A + a_offset(96 + d, k)) = il;
            }
            fence_async_smem();
            __syncthreads();
            if (tid == 0) {
                fence_after_sync();
                for (int kk = 0; kk < (kpad >> 4); ++kk) {
                    const uint64_t desc = make_smem_desc(a_base + kk * 256, 128, TC_SBO);
                    tc_mma(tbase, desc, desc, TC_IDESC, (c0 > 0 || kk > 0) ? 1u : 0u);
                }
                tc_commit(mbar);
            }
            // every thread waits for the MMAs (bounded); the vote keeps the
            // timeout decision uniform across the CTA
            long long spins = 0;
            bool late = false;
            while (!mbar_try_wait(mbar, phase)) {
                if (++spins > TC_SPIN_LIMIT) { late = true; break; }
            }
            timed_out = __syncthreads_or(late) != 0;
            if (timed_out) break;
            phase ^= 1u;
        }
        if (timed_out) {
            if (tid == 0) { atomicOr(P.err, ERR_TC_TIMEOUT); flag[1] = 1; }
            break;
        }
        fence_after_sync();
        // ---- read D: warp w holds TMEM lanes 32w..32w+31 (rows of D) ----
        {
            uint32_t r[16];
            const int row = 32 * warp + lane;
#pragma unroll
            for (int c16 = 0; c16 < 4; ++c16) {
                tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + 16 * c16, r);
                tmem_wait_ld();
#pragma unroll
                for (int j = 0; j < 16; ++j) D[row * TC_LDD + 16 * c16 + j] = __uint_as_float(r[j]);
            }
        }
        fence_before_sync();
        __syncthreads();
        // ---- Gamma, coherence, packed store ----
        // S(a,b) = D[a][b] + D[64+a][b] + D[64+b][a]
        auto S = [&](int a, int b) {
            return D[a * TC_LDD + b] + D[(64 + a) * TC_LDD + b] + D[(64 + b) * TC_LDD + a];
        };
        if (tid < 32) {
            bool bad = false;
            if (tid < n) {
                const float Pi = S(tid, tid) + S(32 + tid, 32 + tid);
                bad = !(Pi > 0.f) || !isfinite(Pi);
                rs[tid] = rsqrtf(Pi);
            }
            bad = __any_sync(0xffffffffu, bad);
            if (tid == 0) flag[0] = bad ? 1 : 0;
        }
        __syncthreads();
        const bool badc = flag[0] != 0;
        if (!badc) {
            // row i of the packed upper triangle starts at i n - i(i-1)/2;
            // warps take rows, lanes take columns j >= i (conflict-free reads)
            float2 *dst = P.cbuf + loc * P.cstride;
            for (int i = warp; i < n; i += 4) {
                const int off = i * n - i * (i - 1) / 2;
                for (int j = i + lane; j < n; j += 32) {
                    float2 c;
                    if (i == j) {
                        c = make_float2(1.f, 0.f);
                    } else {
                        const float re = S(i, j) + S(32 + i, 32 + j);
                        const float im = S(32 + i, j) - S(i, 32 + j);
                        const float sc = rs[i] * rs[j];
                        c = make_float2(re * sc, im * sc);
                        if (!isfinite(c.x) || !isfinite(c.y)) flag[0] = 1;
                    }
                    dst[off + (j - i)] = c;
                }
            }
        }
        __syncthreads();
        if (tid == 0) P.cinfo[loc] = flag[0] ? CI_BAD : npix;
        __syncthreads();
    }
    __syncthreads();
    if (flag[1] && tid == 0) {
        // after a timeout, give the MMAs in flight a second bounded wait
        // before their tensor memory is released
        long long spins = 0;
        while (!mbar_try_wait(mbar, phase) && ++spins < TC_SPIN_LIMIT) {
        }
    }
    __syncthreads();
    fence_after_sync();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(TC_TMEM_COLS) : "memory");
    }
}

}  // namespace

cudaError_t launch_gram_tc(const KParams &P, int num_sms, cudaStream_t st)
{
    static bool configured[64] = {false};
    if (P.nb > 32 || P.K > TC_MAXK) return cudaErrorInvalidValue;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !configured[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        if (e != cudaSuccess) return e;
        configured[dev] = true;
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gram_tc, TC_THREADS, TC_SMEM);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    if (per_sm > 8) per_sm = 8;               // 8 x 64 TMEM columns of the 512
    long long blocks = (long long)num_sms * per_sm;
    if (P.npix < blocks) blocks = P.npix > 0 ? P.npix : 1;
    k_gram_tc<<<(unsigned)blocks, TC_THREADS, TC_SMEM, st>>>(P);
    return cudaGetLastError();
}

}  // namespace fpl
