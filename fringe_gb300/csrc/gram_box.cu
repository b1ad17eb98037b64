// gram_box.cu -- coherence matrices on the 5th-generation tensor cores, one
// tile of 128 pixels per GEMM.
//
// Mixed-precision form of the SHP gather + Gamma accumulation
// (src/evd/evd.cpp:516-564, src/phase_link/phase_link.cpp:482-522).  For a
// pixel p the reference sums x_q x_q^H over its SHPs q.  Written for a tile
// of pixels at once this is a masked box filter of the per-sample outer
// products,
//     Gamma_p = sum_q m_pq x_q x_q^H,   m_pq = 1 iff q is an SHP of p,
// which is a dense GEMM over the samples q of the union of the tile's windows:
//     D[p][c] = sum_q A[p][q] B[c][q]
//   A = the 0/1 SHP mask (exact in bf16), rows = the 128 pixels of an
//       8 x 16 pixel tile, columns = the (8+Wy-1) x (16+Wx-1) union samples;
//   B = the outer-product entries Re / Im x_qi conj(x_qj), formed in FP32
//       (the reference's complex<float> products) and split into bf16
//       hi + lo parts (16 significant bits), so D = A B_hi + A B_lo is
//       accumulated in FP32 in tensor memory.
// Each outer product is formed once per tile instead of once for every pixel
// that uses it.  One thread issues tcgen05.mma (M = 128 pixels, N <= 256
// Gamma entries, K = 16 samples) into one of two tensor-memory accumulators;
// the Gamma entries are processed in passes of 512 columns, each pass over
// the tile's samples in chunks of 32 (two operand stages, one CTA barrier
// per chunk).
//
// Column order (the Gamma record read by the eigen kernel): dates padded to an
// even count and grouped in pairs; block (a, b), a <= b, row-major over the
// upper triangle of pairs, holds 8 floats: Re, Im of Gamma_ij for
// (i, j) = (2a,2b), (2a,2b+1), (2a+1,2b), (2a+1,2b+1).
//
// Operand layout (no swizzle, K-major): core matrices of 8 rows x 16 bytes;
// K-adjacent core matrices 128 B apart, 8-row groups KC*16+16 B apart (the
// 16-byte pad keeps the staging stores free of bank conflicts).
//
// Samples whose value is non-finite, or whose components lie outside
// [2^-50, 2^50] in magnitude (other than 0), are outside the range of the
// split: they are zeroed in the tile and every pixel that has one among its
// SHPs is handed to the FP64 path (CI_DEFER), which follows the reference
// exactly.  Every wait on the tensor core is bounded; on timeout the CTA
// records an error flag, stops, and frees its tensor memory after a second
// bounded wait.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"
#include "pixel.cuh"

namespace fpl {
namespace {

constexpr int BX_THREADS = 512;                    // 16 warps: the operand build hides latency
constexpr int BX_TR = 8, BX_TC = 16, BX_M = 128;   // pixel tile (MMA M)
constexpr int BX_NCOL = 256;                       // Gamma columns per accumulator (MMA N)
// samples per chunk (MMA K of one stage): 32, so that two accumulators (512
// Gamma columns per pass) fit beside two operand stages and two sample buffers
constexpr int BX_KC = 32;
constexpr int BX_MAXK = 2048;                      // union samples per tile
constexpr int BX_MAXW = BX_MAXK / 32;              // union mask words per pixel
constexpr int BX_MAXWX = 63;                       // window width (64-bit row extraction)
constexpr int BX_MISC = 4096;
constexpr int CI_SKIP = -100;                      // pixel outside this launch's rows
constexpr unsigned ERR_TC_TIMEOUT = 2u;
constexpr long long BX_SPIN_LIMIT = 1ll << 26;     // ~ seconds of polling

template <int KC> struct BoxLay {
    // tensor-memory accumulators of BX_NCOL columns each: with 32-sample
    // chunks two fit beside two operand stages, so a pass covers 512 Gamma
    // columns and a chunk's samples and mask are loaded and built once for
    // both
    static constexpr int NACC = (KC == 32) ? 2 : 1;
    static constexpr int PCOL = NACC * BX_NCOL;               // Gamma columns per pass
    static constexpr int SBO = KC * 16 + 16;                 // bytes between 8-row groups
    static constexpr int A_BYTES = (BX_M / 8) * SBO;
    static constexpr int B_BYTES = (PCOL / 8) * SBO;         // one of hi / lo
    static constexpr int STAGE = A_BYTES + 2 * B_BYTES;
    static constexpr int MAXPAIR = 32;                       // date pairs: 64 dates
    static constexpr int XRS = KC * 16 + 16;                 // bytes per date-pair row of X
    static constexpr int X_BYTES = MAXPAIR * XRS;            // one of two sample buffers
    static constexpr size_t OFF_X = 2 * (size_t)STAGE;
    static constexpr size_t OFF_MISC = OFF_X + 2 * (size_t)X_BYTES;
    static constexpr size_t OFF_LUT = OFF_MISC + BX_MISC;          // 256 x 8 bf16 mask patterns
    static constexpr size_t OFF_U = OFF_LUT + 256 * 16;
    static constexpr size_t MAX_SMEM = OFF_U + (size_t)BX_M * BX_MAXW * 4;
    static_assert(MAX_SMEM <= 227 * 1024, "shared memory of one CTA");
};

// union samples of a tile: (8 + 2 ny) rows of (16 + 2 nx) samples, packed
// row after row (no padding: every sample slot is a GEMM K index)
__host__ __device__ __forceinline__ int box_union_cols(int nx) { return BX_TC + 2 * nx; }

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
// K-major, M = 128, N = n
__device__ __forceinline__ uint32_t make_idesc(int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((128u >> 4) << 24);
}

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

// 32 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t *r)
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// len (<= 63) bits of a little-endian word array starting at bit pos
__device__ __forceinline__ uint64_t extract_bits(const uint32_t *w, int nul, int pos, int len)
{
    const int w0 = pos >> 5, sh = pos & 31;
    uint64_t v = w[w0];
    if (w0 + 1 < nul) v |= (uint64_t)w[w0 + 1] << 32;
    v >>= sh;
    if (sh && w0 + 2 < nul) v |= (uint64_t)w[w0 + 2] << (64 - sh);
    return v & ((1ull << len) - 1ull);
}

// 0 or a normal magnitude in [2^-50, 2^50]: the bf16 split of every product
// of two such components stays normal and the window sums stay finite
__device__ __forceinline__ bool split_range(float v)
{
    const float a = fabsf(v);
    return v == 0.f || (a >= 8.8817842e-16f && a <= 1.1258999e15f);
}

// 8 values of one Gamma column into bf16 hi and lo rows (16 bytes each)
__device__ __forceinline__ void store_split(unsigned char *dh, unsigned char *dl, const float *v)
{
    uint32_t h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const __nv_bfloat162 hb = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
        const uint32_t hu = *reinterpret_cast<const uint32_t *>(&hb);
        const float h0 = __uint_as_float(hu << 16), h1 = __uint_as_float(hu & 0xffff0000u);
        const __nv_bfloat162 lb = __floats2bfloat162_rn(v[2 * q] - h0, v[2 * q + 1] - h1);
        h[q] = hu;
        l[q] = *reinterpret_cast<const uint32_t *>(&lb);
    }
    *reinterpret_cast<uint4 *>(dh) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(dl) = make_uint4(l[0], l[1], l[2], l[3]);
}

// pipeline state of a CTA, carried from tile to tile (and job to job)
struct BoxPipe {
    uint32_t pend;      // per stage: MMAs in flight
    uint32_t par;       // per stage: mbarrier parity
    unsigned gstep;     // chunks issued
    bool timed_out;
    int blk_dp;         // date pairs the block table was built for
};

// this thread's wait for the MMAs of stage s (if any are pending); true if
// the wait gave up.  Every thread polls the barrier itself, so no CTA
// barrier is needed before the stage is overwritten.
__device__ __forceinline__ bool box_poll(uint64_t *mbar, BoxPipe &st, int s)
{
    if (!(st.pend & (1u << s))) return false;
    long long spins = 0;
    while (!mbar_try_wait(&mbar[s], (st.par >> s) & 1u))
        if (++spins > BX_SPIN_LIMIT) return true;
    st.par ^= 1u << s;
    st.pend &= ~(1u << s);
    return false;
}

// tiles of the rows [ra, rb) of a launch: 8-row tiles on the absolute grid
// (rows 8t .. 8t+7 of the scene) so that a pixel's Gamma, and its order of
// accumulation, do not depend on how the rows were split into launches
__device__ __forceinline__ int box_first_row(const KParams &P) { return int(P.pix_begin / P.cols) / BX_TR * BX_TR; }
__host__ __device__ __forceinline__ long long box_tiles(const KParams &P)
{
    const int ra = int(P.pix_begin / P.cols), rb = ra + int(P.npix / P.cols);
    if (rb <= ra) return 0;
    const int r0 = ra / BX_TR * BX_TR;
    return (long long)((P.cols + BX_TC - 1) / BX_TC) * ((rb - r0 + BX_TR - 1) / BX_TR);
}

// Gamma records of tile t of the launch described by P (all threads of the
// CTA call it together)
template <int KC>
__device__ void box_tile(const KParams &P, long long t, unsigned char *smem, uint32_t tbase, BoxPipe &st)
{
    using L = BoxLay<KC>;
    unsigned char *Xb = smem + L::OFF_X;
    unsigned char *misc = smem + L::OFF_MISC;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(misc);                 // 2 stages
    int *pinfo = reinterpret_cast<int *>(misc + 64);                     // 128
    int *pdefer = reinterpret_cast<int *>(misc + 64 + 512);              // 128
    short2 *blk = reinterpret_cast<short2 *>(misc + 64 + 1024);          // <= 528 blocks
    uint32_t *tbad = reinterpret_cast<uint32_t *>(misc + 3200);          // [W] out-of-range samples
    uint32_t *umask = reinterpret_cast<uint32_t *>(smem + L::OFF_U);     // [128][W]
    const uint4 *lut = reinterpret_cast<const uint4 *>(smem + L::OFF_LUT);
    uint32_t *nm = reinterpret_cast<uint32_t *>(smem + L::STAGE);        // nmap words (stage 1, mask build only)

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = P.nb, dp = (n + 1) >> 1, nblk = dp * (dp + 1) / 2, ncolt = 8 * nblk;
    const int cols = P.cols, rows = P.rows, nul = P.nulong;
    const int wy = 2 * P.ny + 1, wx = P.wx;
    const int uh = BX_TR + wy - 1, uwp = box_union_cols(P.nx);   // union rows, columns
    const int kp = (uh * uwp + KC - 1) / KC * KC, nchunk = kp / KC;
    const int W = kp >> 5;
    const int ra = int(P.pix_begin / cols), rb = ra + int(P.npix / cols);
    const int ntc = (cols + BX_TC - 1) / BX_TC;
    const int npass = (ncolt + L::PCOL - 1) / L::PCOL;
    const int min_neigh = (P.semantics == SEM_PL) ? P.min_neigh : 2;   // evd.cpp:566
    const long long plane = P.plane;
    const int R0 = box_first_row(P) + int(t / ntc) * BX_TR, C0 = int(t % ntc) * BX_TC;

    // Gamma column blocks (a, b), a <= b, of this stack depth
    if (st.blk_dp != dp) {
        __syncthreads();
        for (int b = tid; b < nblk; b += BX_THREADS) {
            int a = 0, rem = b;
            while (rem >= dp - a) { rem -= dp - a; ++a; }
            blk[b] = make_short2((short)a, (short)(a + rem));
        }
        st.blk_dp = dp;
    }
    // ---- per-pixel SHP masks over the union samples ----------------
    for (int e = tid; e < BX_M * W; e += BX_THREADS) umask[e] = 0;
    for (int e = tid; e < W; e += BX_THREADS) tbad[e] = 0;
    for (int e = tid; e < BX_M * nul; e += BX_THREADS) {
        const int m = e / nul, w = e - m * nul;
        const int r = R0 + m / BX_TC, c = C0 + m % BX_TC;
        nm[e] = (r >= ra && r < rb && c < cols) ? __ldg(P.nmap + ((long long)r * cols + c) * nul + w) : 0u;
    }
    __syncthreads();
    for (int e = tid; e < BX_M * wy; e += BX_THREADS) {
        const int m = e / wy, a = e - m * wy;
        const int tr = m / BX_TC, tc = m % BX_TC;
        const int r = R0 + tr, c = C0 + tc;
        const int sr = r - P.ny + a;                    // image row of window row a
        if (r < ra || r >= rb || c >= cols || sr < 0 || sr >= rows) continue;
        uint64_t bits = extract_bits(nm + m * nul, nul, a * wx, wx);
        // window column b is image column c - nx + b (evd.cpp:530-534)
        const int blo = max(0, P.nx - c), bhi = min(wx, cols - c + P.nx);
        if (bhi <= blo) continue;
        bits &= ((1ull << (bhi - blo)) - 1ull) << blo;
        if (!bits) continue;
        const int pos = (tr + a) * uwp + tc;            // union sample of window (a, 0)
        const int w0 = pos >> 5, sh = pos & 31;
        const uint64_t lo = bits << sh;
        const uint32_t hi = sh ? (uint32_t)(bits >> (64 - sh)) : 0u;
        uint32_t *um = umask + m * W;
        if ((uint32_t)lo) atomicOr(um + w0, (uint32_t)lo);
        if ((uint32_t)(lo >> 32)) atomicOr(um + w0 + 1, (uint32_t)(lo >> 32));
        if (hi) atomicOr(um + w0 + 2, hi);
    }
    __syncthreads();
    if (tid < BX_M) {
        const int m = tid, r = R0 + m / BX_TC, c = C0 + m % BX_TC;
        int info = CI_SKIP;                                 // outside rows [ra, rb) of this launch
        if (r >= ra && r < rb && c < cols) {
            const int cflat = P.ny * wx + P.nx;
            if (!((nm[m * nul + (cflat >> 5)] >> (cflat & 31)) & 1u)) {
                info = CI_CENTRE;                       // evd.cpp:517
            } else {
                int cnt = 0;
                for (int w = 0; w < W; ++w) cnt += __popc(umask[m * W + w]);
                info = (cnt < min_neigh) ? CI_FEW : cnt;
            }
        }
        pinfo[m] = info;
    }
    // (the prologue's barrier orders these before any use)

    // samples of chunk k0 (date pairs interleaved): each thread loads one
    // sample for up to BX_XPT dates into registers (64 dates over the CTA);
    // put() stores them in one of two sample buffers (chunk g in buffer
    // g & 1) and flags samples outside the split range in tbad.  The loads
    // run two chunks ahead of the build: chunk c waits in xa (c even) or xb
    // (c odd), chosen by a branch so both stay in registers, and no copy
    // between them waits for loads in flight.
    constexpr int BX_XPT = 2 * L::MAXPAIR * KC / BX_THREADS;
    static_assert(BX_XPT >= 1 && BX_XPT * (BX_THREADS / KC) == 2 * L::MAXPAIR, "date coverage");
    const int sidx = tid % KC, d0 = tid / KC;
    float2 xa[BX_XPT], xb[BX_XPT];
    // chunks are loaded in cyclic order (0, 1, .., nchunk - 1, 0, ..): the
    // union row and column of this thread's next sample advance by KC
    // (< 3 union rows of >= 16 samples) and return to the start after the
    // last chunk, with no division per chunk
    const int ur0 = sidx / uwp, uc0 = sidx - ur0 * uwp;
    int fur = ur0, fuc = uc0, fch = 0;
    const float2 *sbase = P.stack + (long long)d0 * plane;
    auto fetch = [&](float2 (&xo)[BX_XPT]) {
        const int r = R0 - P.ny + fur, c = C0 - P.nx + fuc;
        const bool valid = fur < uh && r >= 0 && r < rows && c >= 0 && c < cols;
        const float2 *src = sbase + (valid ? (long long)r * cols + c : 0ll);
#pragma unroll
        for (int q = 0; q < BX_XPT; ++q) {
            const int d = d0 + q * (BX_THREADS / KC);
            float2 x = make_float2(0.f, 0.f);
            if (valid && d < n) x = __ldg(src + (long long)(q * (BX_THREADS / KC)) * plane);
            xo[q] = x;
        }
        if (++fch == nchunk) {
            fch = 0;
            fur = ur0;
            fuc = uc0;
        } else {
            fuc += KC;
            if (fuc >= uwp) { fuc -= uwp; ++fur; }
            if (fuc >= uwp) { fuc -= uwp; ++fur; }
        }
    };
    // range checks: always in the first pass; in later passes only if the
    // first found an out-of-range sample in the tile (clean: it found none)
    bool clean = false;
    auto put = [&](unsigned char *xd, int k0, const float2 (&xv)[BX_XPT]) {
        bool xbad = false;
#pragma unroll
        for (int q = 0; q < BX_XPT; ++q) {
            const int d = d0 + q * (BX_THREADS / KC);
            if (d >= 2 * dp) break;
            float2 x = xv[q];
            if (!clean && (!split_range(x.x) || !split_range(x.y))) {
                xbad = true;
                x = make_float2(0.f, 0.f);
            }
            *reinterpret_cast<float2 *>(xd + (d >> 1) * L::XRS + sidx * 16 + (d & 1) * 8) = x;
        }
        if (xbad) atomicOr(tbad + ((k0 + sidx) >> 5), 1u << ((k0 + sidx) & 31));
    };
    static_assert(KC <= 2 * BX_TC, "a chunk advances at most two union rows");
    // prologue: the first chunk of the tile into buffer 0, the second one
    // into xb
    const int gtot = npass * nchunk;
    fetch(xa);
    put(Xb, 0, xa);
    if (gtot > 1) fetch(xb);
    __syncthreads();

    for (int pass = 0; pass < npass && !st.timed_out; ++pass) {
        const int cb = pass * L::PCOL;
        const int ncol = min(L::PCOL, ncolt - cb);
        // accumulator j holds the pass's columns [256 j, 256 j + 256)
        int nmma[L::NACC];
        uint32_t idesc[L::NACC];
#pragma unroll
        for (int j = 0; j < L::NACC; ++j) {
            const int nc = min(BX_NCOL, ncol - j * BX_NCOL);
            nmma[j] = nc > 0 ? (nc + 15) & ~15 : 0;
            idesc[j] = make_idesc(nmma[j] > 0 ? nmma[j] : 16);
        }
        for (int ch = 0; ch < nchunk; ++ch) {
            const int s = st.gstep & 1;
            // the stage's previous MMAs (two chunks back) must be done
            // before it is overwritten; a thread whose wait gave up builds
            // nothing and the vote below stops the CTA
            const bool late = box_poll(mbar, st, s);
            unsigned char *As = smem + s * L::STAGE;
            unsigned char *Bh = As + L::A_BYTES, *Bl = Bh + L::B_BYTES;
            const int k0 = ch * KC;
            // chunk g + 1 (the first chunk again after the last one of a
            // pass) is in registers; chunk g + 2 is loaded while this one
            // is built, into the array chunk g left
            const int g = pass * nchunk + ch;
            const bool more = g + 1 < gtot;
            const unsigned char *Xc = Xb + (g & 1) * L::X_BYTES;
            if (g + 2 < gtot) {
                if (g & 1) fetch(xb);
                else fetch(xa);
            }
            // ---- A: SHP mask rows ----
            for (int e = late ? BX_M * (KC / 8) : tid; e < BX_M * (KC / 8); e += BX_THREADS) {
                const int m = e & (BX_M - 1), k8 = e >> 7;
                const int b0 = k0 + k8 * 8;
                const uint32_t bits = (umask[m * W + (b0 >> 5)] >> (b0 & 31)) & 0xffu;
                *reinterpret_cast<uint4 *>(As + (m >> 3) * L::SBO + k8 * 128 + (m & 7) * 16) = lut[bits];
            }
            // ---- B: outer-product entries, hi and lo ----
            // one thread per half core matrix: block bl's rows 4 ia .. 4 ia + 3
            // (entries (2a + ia, 2b), (2a + ia, 2b + 1), Re and Im) over the 8
            // samples of K group k8
            constexpr int NBL = L::PCOL / 8;                 // column blocks of the pass
            for (int e = late ? 2 * NBL * (KC / 8) : tid; e < 2 * NBL * (KC / 8); e += BX_THREADS) {
                const int bl = e % NBL, ia = (e / NBL) & 1, k8 = e / (2 * NBL);
                const int jacc = bl / (BX_NCOL / 8);
                const int nm_j = (jacc == 0) ? nmma[0] : nmma[L::NACC - 1];
                if ((bl - jacc * (BX_NCOL / 8)) * 8 >= nm_j) continue;          // read by no MMA
                unsigned char *dh = Bh + bl * L::SBO + k8 * 128 + ia * 64;
                unsigned char *dl = Bl + bl * L::SBO + k8 * 128 + ia * 64;
                if (bl * 8 >= ncol) {
                    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        *reinterpret_cast<uint4 *>(dh + c * 16) = z;
                        *reinterpret_cast<uint4 *>(dl + c * 16) = z;
                    }
                    continue;
                }
                const short2 ab = blk[cb / 8 + bl];
                const unsigned char *sa = Xc + ab.x * L::XRS + k8 * 128;
                const unsigned char *sb = Xc + ab.y * L::XRS + k8 * 128;
                float2 pa[8];          // per sample: x_{2a + ia}
                float4 pb[8];          // per sample: x_{2b}, x_{2b+1}
#pragma unroll
                for (int q = 0; q < 8; ++q) pa[q] = *reinterpret_cast<const float2 *>(sa + q * 16 + ia * 8);
#pragma unroll
                for (int q = 0; q < 8; ++q) pb[q] = *reinterpret_cast<const float4 *>(sb + q * 16);
#pragma unroll
                for (int jb = 0; jb < 2; ++jb) {           // i = 2a + ia, j = 2b + jb
                    float re[8], im[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const float xr = pa[q].x, xi = pa[q].y;
                        const float yr = jb ? pb[q].z : pb[q].x, yi = jb ? pb[q].w : pb[q].y;
                        re[q] = fmaf(xr, yr, xi * yi);          // Re x_i conj(x_j)
                        im[q] = fmaf(xi, yr, -(xr * yi));       // Im x_i conj(x_j)
                    }
                    store_split(dh + (2 * jb) * 16, dl + (2 * jb) * 16, re);
                    store_split(dh + (2 * jb + 1) * 16, dl + (2 * jb + 1) * 16, im);
                }
            }
            // the next chunk's samples go to the other buffer, which the
            // previous chunk's build (before the previous barrier) read last
            if (more) {
                unsigned char *Xn = Xb + ((g + 1) & 1) * L::X_BYTES;
                const int kn = ((g + 1) % nchunk) * KC;
                if (g & 1) put(Xn, kn, xa);
                else put(Xn, kn, xb);
            }
            fence_async_smem();
            if (__syncthreads_or(late)) { st.timed_out = true; break; }
            if (tid == 0) {
                fence_after_sync();
                const uint32_t a0 = smem_addr(As), h0 = smem_addr(Bh), l0 = smem_addr(Bl);
#pragma unroll
                for (int kk = 0; kk < KC / 16; ++kk) {
                    const uint64_t da = make_smem_desc(a0 + kk * 256, 128, L::SBO);
#pragma unroll
                    for (int j = 0; j < L::NACC; ++j) {
                        if (nmma[j] == 0) continue;
                        const uint32_t boff = (uint32_t)(j * (BX_NCOL / 8) * L::SBO + kk * 256);
                        const uint64_t dh = make_smem_desc(h0 + boff, 128, L::SBO);
                        const uint64_t dl = make_smem_desc(l0 + boff, 128, L::SBO);
                        const uint32_t dt = tbase + (uint32_t)(j * BX_NCOL);
                        tc_mma(dt, da, dh, idesc[j], (ch > 0 || kk > 0) ? 1u : 0u);
                        tc_mma(dt, da, dl, idesc[j], 1u);
                    }
                }
                tc_commit(&mbar[s]);
            }
            st.pend |= 1u << s;
            ++st.gstep;
        }
        if (st.timed_out) return;
        const bool late = box_poll(mbar, st, 0) || box_poll(mbar, st, 1);
        if (pass == 0 && tid < BX_M) {
            // every sample of the tile has been stored (the last one before
            // the last chunk's barrier): a pixel with an out-of-range SHP
            // sample goes to the FP64 path
            const int m = tid;
            uint32_t hit = 0;
            for (int w = 0; w < W; ++w) hit |= umask[m * W + w] & tbad[w];
            pdefer[m] = hit != 0;
        }
        if (__syncthreads_or(late)) { st.timed_out = true; break; }
        fence_after_sync();
        if (pass == 0) {
            uint32_t any = 0;
            for (int w = 0; w < W; ++w) any |= tbad[w];
            clean = any == 0;
        }
        // ---- epilogue: warp w reads TMEM lanes 32(w%4).., BX_CPW x 32 columns ----
        // A lane holds its own pixel's columns; they are written out through
        // a 32 x 32 staging tile per warp (in the operand stages, which no
        // MMA reads any more: both stages were waited for above) so that
        // each store instruction writes four pixels' 128 contiguous bytes
        // instead of 32 pixels' 16.
        {
            constexpr int BX_CPW = (L::PCOL / 32) / (BX_THREADS / 128);
            constexpr int SROW = 36;                        // staging row stride (floats)
            static_assert((BX_THREADS / 32) * 32 * SROW * 4 <= 2 * L::STAGE, "staging fits the stages");
            float *stg = reinterpret_cast<float *>(smem) + warp * (32 * SROW);
            float *rec = reinterpret_cast<float *>(P.cbuf);
            const int q = warp & 3, h = warp >> 2;
            for (int c32 = BX_CPW * h; c32 < BX_CPW * h + BX_CPW; ++c32) {
                const int col0 = 32 * c32;
                if (col0 >= ncol) break;
                uint32_t v[32];
                tmem_ld32(tbase + ((uint32_t)(32 * q) << 16) + (uint32_t)col0, v);
                tmem_wait_ld();
#pragma unroll
                for (int j = 0; j < 32; j += 4)
                    *reinterpret_cast<float4 *>(stg + lane * SROW + j) =
                        make_float4(__uint_as_float(v[j]), __uint_as_float(v[j + 1]),
                                    __uint_as_float(v[j + 2]), __uint_as_float(v[j + 3]));
                __syncwarp();
                const int lim = min(32, ncol - col0);
                const int j = 4 * (lane & 7);
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int pl = 4 * i + (lane >> 3);          // pixel of the warp's 32
                    const int m = 32 * q + pl;
                    if (j < lim && pinfo[m] >= 0 && !pdefer[m]) {
                        const long long loc = (long long)(R0 + m / BX_TC) * cols + (C0 + m % BX_TC) - P.cbase;
                        *reinterpret_cast<float4 *>(rec + loc * P.cstride + cb + col0 + j) =
                            *reinterpret_cast<const float4 *>(stg + pl * SROW + j);
                    }
                }
                __syncwarp();
            }
        }
        fence_before_sync();
        __syncthreads();
    }
    if (st.timed_out) return;
    if (tid < BX_M) {
        const int m = tid, info = pinfo[m];
        if (info != CI_SKIP) {
            const long long loc = (long long)(R0 + m / BX_TC) * cols + (C0 + m % BX_TC) - P.cbase;
            P.cinfo[loc] = (info >= 0 && pdefer[m]) ? CI_DEFER : info;
        }
    }
    __syncthreads();

}

template <int KC>
__device__ __forceinline__ uint32_t box_setup(unsigned char *smem, BoxPipe &st)
{
    using L = BoxLay<KC>;
    unsigned char *misc = smem + L::OFF_MISC;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(misc);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(misc + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(tmem_slot)), "r"(L::PCOL) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // mask patterns: entry b holds 8 bf16 values, 1 where bit q of b is set
    uint4 *lut = reinterpret_cast<uint4 *>(smem + L::OFF_LUT);
    for (int b = tid; b < 256; b += BX_THREADS) {
        uint32_t v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            v[q] = ((b >> (2 * q)) & 1 ? 0x3F80u : 0u) | ((b >> (2 * q + 1)) & 1 ? 0x3F800000u : 0u);
        lut[b] = make_uint4(v[0], v[1], v[2], v[3]);
    }
    st.pend = 0;
    st.par = 0;
    st.gstep = 0;
    st.timed_out = false;
    st.blk_dp = -1;
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    return *tmem_slot;
}

// on a timeout: record the error, give the MMAs in flight a second bounded
// wait; then release the tensor memory
template <int KC>
__device__ __forceinline__ void box_teardown(unsigned char *smem, uint32_t tbase, BoxPipe &st, unsigned *err)
{
    using L = BoxLay<KC>;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::OFF_MISC);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (st.timed_out) {
        if (tid == 0) atomicOr(err, ERR_TC_TIMEOUT);
        for (int s = 0; s < 2; ++s) {
            if (st.pend & (1u << s)) {
                long long spins = 0;
                while (!mbar_try_wait(&mbar[s], (st.par >> s) & 1u) && ++spins < BX_SPIN_LIMIT) {
                }
            }
        }
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(L::PCOL) : "memory");
    }
}

template <int KC>
__global__ void __launch_bounds__(BX_THREADS, 1) k_gram_box(KParams P)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    BoxPipe st;
    const uint32_t tbase = box_setup<KC>(smem, st);
    const long long ntiles = box_tiles(P);
    for (long long t = blockIdx.x; t < ntiles && !st.timed_out; t += gridDim.x)
        box_tile<KC>(P, t, smem, tbase, st);
    box_teardown<KC>(smem, tbase, st, P.err);
}

// Many launches' tiles in one persistent launch: segment s covers tiles
// [segs[s].tile_offset, segs[s+1].tile_offset) of the concatenation.
template <int KC>
__global__ void __launch_bounds__(BX_THREADS, 1) k_gram_batch(const BoxSeg *__restrict__ segs, int nseg,
                                                              long long total)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    BoxPipe st;
    const uint32_t tbase = box_setup<KC>(smem, st);
    for (long long t = blockIdx.x; t < total && !st.timed_out; t += gridDim.x) {
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (segs[mid].tile_offset <= t) lo = mid; else hi = mid - 1;
        }
        box_tile<KC>(segs[lo].P, t - segs[lo].tile_offset, smem, tbase, st);
    }
    box_teardown<KC>(smem, tbase, st, segs[0].P.err);
}

template <int KC>
size_t box_smem(int ny, int nx)
{
    using L = BoxLay<KC>;
    const int uh = BX_TR + 2 * ny, uwp = box_union_cols(nx);
    const int kp = (uh * uwp + KC - 1) / KC * KC;
    return L::OFF_U + (size_t)BX_M * (kp / 32) * 4;
}

// per-kernel flags: attributes set once per device
template <int KC, bool BATCH>
bool *box_flags()
{
    static bool f[64] = {false};
    return f;
}

template <typename K>
cudaError_t box_configure(K kern, size_t smem_max, bool *configured)
{
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && configured[dev]) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
    if (e == cudaSuccess && dev < 64) configured[dev] = true;
    return e;
}

template <int KC>
cudaError_t launch_box_t(const KParams &P, int num_sms, cudaStream_t st)
{
    using L = BoxLay<KC>;
    cudaError_t e = box_configure(k_gram_box<KC>, L::MAX_SMEM, box_flags<KC, false>());
    if (e != cudaSuccess) return e;
    const long long ntiles = box_tiles(P);
    long long blocks = num_sms;
    if (ntiles < blocks) blocks = ntiles > 0 ? ntiles : 1;
    k_gram_box<KC><<<(unsigned)blocks, BX_THREADS, box_smem<KC>(P.ny, P.nx), st>>>(P);
    return cudaGetLastError();
}

template <int KC>
cudaError_t launch_box_batch_t(const BoxSeg *segs, int nseg, long long total, size_t smem, int num_sms,
                               cudaStream_t st)
{
    using L = BoxLay<KC>;
    cudaError_t e = box_configure(k_gram_batch<KC>, L::MAX_SMEM, box_flags<KC, true>());
    if (e != cudaSuccess) return e;
    long long blocks = num_sms;
    if (total < blocks) blocks = total > 0 ? total : 1;
    k_gram_batch<KC><<<(unsigned)blocks, BX_THREADS, smem, st>>>(segs, nseg, total);
    return cudaGetLastError();
}

}  // namespace

bool gram_box_supported(int nb, int ny, int nx)
{
    const int wx = 2 * nx + 1;
    if (nb < 1 || nb > 64 || wx > BX_MAXWX) return false;
    const int uh = BX_TR + 2 * ny, uwp = box_union_cols(nx);
    return (long long)uh * uwp <= BX_MAXK;
}

int gram_box_record(int nb)
{
    const int dp = (nb + 1) >> 1;
    return 8 * (dp * (dp + 1) / 2);
}

long long gram_box_tiles(const KParams &P) { return box_tiles(P); }

size_t gram_box_smem(int nb, int ny, int nx)
{
    (void)nb;
    return box_smem<BX_KC>(ny, nx);
}

cudaError_t prepare_gram_batch()
{
    return box_configure(k_gram_batch<BX_KC>, BoxLay<BX_KC>::MAX_SMEM, box_flags<BX_KC, true>());
}

cudaError_t launch_gram_batch(const BoxSeg *segs, int nseg, long long total, size_t smem, int num_sms,
                              cudaStream_t st)
{
    if (nseg <= 0 || total <= 0) return cudaSuccess;
    return launch_box_batch_t<BX_KC>(segs, nseg, total, smem, num_sms, st);
}

cudaError_t launch_gram_box(const KParams &P, int num_sms, cudaStream_t st)
{
    if (!gram_box_supported(P.nb, P.ny, P.nx) || P.cols <= 0 || P.pix_begin % P.cols || P.npix % P.cols)
        return cudaErrorInvalidValue;
    if (P.npix == 0) return cudaSuccess;
    return launch_box_t<BX_KC>(P, num_sms, st);
}

}  // namespace fpl
