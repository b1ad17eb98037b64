// batch.cu -- many phase-linking jobs in one persistent launch.
//
// A batch holds device-memory jobs of different scene sizes, stack depths
// (ministacks of different N), windows and methods.  Jobs whose padded depth
// NP matches share one persistent kernel: warps take pixels from a global
// counter over the concatenated pixel ranges of the jobs (dynamic scheduling
// balances tiles of uneven size and uneven SHP counts), look up the pixel's
// job and run the same per-pixel code as fpl_run.  A second persistent
// kernel settles, in FP64, the pixels every job queued.  The whole sequence
// (counter resets and the kernels of every depth class) can be captured once
// into a CUDA graph and replayed.
//
// Jobs in the mixed-precision form (fpl_job::precision = FPL_PREC_MIXED) are
// cut into row pieces and packed into waves of at most 2^20 pixels; a wave
// is one persistent tensor-core Gamma launch over the tiles of all its
// pieces and one persistent solve launch over all
// its pixels (per padded depth), the Gamma records staying in a buffer
// sized for one wave.  Their FP64 settle runs with the FP32 jobs' at the end.
//
// An optional autotuner times the candidate CTA shapes (warps per CTA) of
// each depth class -- the FP32 batch launches and the mixed form's solve
// launches -- on the batch itself and keeps the fastest per (form, NP,
// window taps, mean SHP count) key in the context.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "batch.h"
#include "ctx.h"
#include "fringe_gb300.h"
#include "guard.h"
#include "kernels.h"
#include "pixel.cuh"

namespace fpl {

constexpr int kBatchChunk = 2;   // pixels a warp takes per counter increment

template <int NP>
__global__ void k_batch(const BatchEntry *__restrict__ jobs, int njobs, long long total,
                        unsigned long long *counter)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *sm = smem + (size_t)warp * KPixWarp<float, NP>::bytes;
    // <= 32 dates: the coherence rows in tensor memory (CRowsTmemF)
    __shared__ uint32_t tslot;
    uint32_t tbase = 0, taddr = 0;
    int tcols = 0;
    if constexpr (CRowsTmemF<float, NP>::value) {
        tcols = tmem_cols_for(warps, NP);
        tbase = tmem_alloc_cta(&tslot, warp, (uint32_t)tcols);
        taddr = tbase + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(warp >> 2) * CRowsTmem<NP>::kColsPerWarp;
    }
    while (true) {
        unsigned long long g = 0;
        if (lane == 0) g = atomicAdd(counter, (unsigned long long)kBatchChunk);
        g = __shfl_sync(0xffffffffu, g, 0);
        if ((long long)g >= total) break;
        const long long end = min((long long)g + kBatchChunk, total);
        for (long long q = (long long)g; q < end; ++q) {
            int lo = 0, hi = njobs - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (jobs[mid].px_offset <= q) lo = mid; else hi = mid - 1;
            }
            const KParams &P = jobs[lo].P;
            process_pixel<float, NP>(P, P.pix_begin + (q - jobs[lo].px_offset), sm, lane, taddr);
        }
    }
    if constexpr (CRowsTmemF<float, NP>::value) tmem_free_cta(tbase, warp, (uint32_t)tcols);
}

template <int NP>
__global__ void k_batch_fp64(const BatchEntry *__restrict__ jobs, int njobs)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *sm = smem + (size_t)warp * Lay<double, NP>::bytes;
    __shared__ uint32_t tslot;
    uint32_t tbase = 0, taddr = 0;
    if constexpr (CInTmem<double, NP>::value) {
        tbase = tmem_alloc_cta(&tslot, warp, 512);
        taddr = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
    }
    for (int j = 0; j < njobs; ++j) {
        const KParams &P = jobs[j].P;
        int cnt = *((volatile int *)P.fb_count);
        cnt = cnt < P.fb_cap ? cnt : P.fb_cap;
        for (long long q = fb_next(P, lane); q < cnt; q = fb_next(P, lane))
            process_pixel<double, NP>(P, P.fb_list[q], sm, lane, taddr);
    }
    if constexpr (CInTmem<double, NP>::value) tmem_free_cta(tbase, warp, 512);
}

__global__ void k_popcount(const uint32_t *__restrict__ w, long long nwords, unsigned long long *sum)
{
    unsigned long long s = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nwords;
         i += (long long)gridDim.x * blockDim.x)
        s += __popc(w[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, s);
}

namespace {
template <typename KernelFn>
cudaError_t configure(KernelFn k, size_t smem)
{
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

template <int NP>
size_t warp_bytes_f32() { return KPixWarp<float, NP>::bytes; }

// shared memory of a k_batch<NP> CTA of `warps` warps: with the coherence
// rows in tensor memory at least half of it, so that one CTA runs per SM and
// none waits on a tensor-memory allocation
template <int NP>
size_t batch_smem_f32(int warps)
{
    const size_t s = KPixWarp<float, NP>::bytes * warps;
    return CRowsTmemF<float, NP>::value ? std::max<size_t>(s, 112 * 1024 + 1024) : s;
}
template <int NP>
size_t warp_bytes_f64() { return Lay<double, NP>::bytes; }

size_t warp_bytes(int np, bool fp64)
{
    switch (np) {
    case 16: return fp64 ? warp_bytes_f64<16>() : warp_bytes_f32<16>();
    case 32: return fp64 ? warp_bytes_f64<32>() : warp_bytes_f32<32>();
    case 64: return fp64 ? warp_bytes_f64<64>() : warp_bytes_f32<64>();
    }
    return 0;
}

}  // namespace

int max_warps(int np, bool fp64)
{
    const size_t per = warp_bytes(np, fp64);
    int w = per ? int((224 * 1024) / per) : 1;
    if (fp64 && np == 64) w = std::min(w, 4);   // C in tensor memory: one lane quadrant per warp
    return std::max(1, std::min(w, 16));
}

template <int NP>
cudaError_t launch_batch_np(const BatchEntry *jobs, int njobs, long long total, unsigned long long *counter,
                            int warps, int num_sms, cudaStream_t st)
{
    const size_t smem = batch_smem_f32<NP>(warps);
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<NP>, warps * 32, smem);
    if (e != cudaSuccess) return e;
    per_sm = std::max(per_sm, 1);
    if (CRowsTmemF<float, NP>::value) per_sm = 1;
    k_batch<NP><<<num_sms * per_sm, warps * 32, smem, st>>>(jobs, njobs, total, counter);
    return cudaGetLastError();
}

template <int NP>
cudaError_t launch_batch64_np(const BatchEntry *jobs, int njobs, int num_sms, cudaStream_t st)
{
    // warps per CTA: shared memory's limit, and no more threads than the
    // kernel's registers allow in one CTA
    cudaFuncAttributes fa;
    cudaError_t ea = cudaFuncGetAttributes(&fa, k_batch_fp64<NP>);
    if (ea != cudaSuccess) return ea;
    const int warps = std::max(1, std::min(max_warps(NP, true), fa.maxThreadsPerBlock / 32));
    const size_t smem = Lay<double, NP>::bytes * warps;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_fp64<NP>, warps * 32, smem);
    if (e != cudaSuccess) return e;
    per_sm = std::max(per_sm, 1);
    k_batch_fp64<NP><<<num_sms * per_sm, warps * 32, smem, st>>>(jobs, njobs);
    return cudaGetLastError();
}

cudaError_t configure_np(int np)
{
    cudaError_t e = cudaSuccess;
    switch (np) {
    case 16:
        e = configure(k_batch<16>, batch_smem_f32<16>(max_warps(16, false)));
        if (e == cudaSuccess) e = configure(k_batch_fp64<16>, Lay<double, 16>::bytes * max_warps(16, true));
        break;
    case 32:
        e = configure(k_batch<32>, batch_smem_f32<32>(max_warps(32, false)));
        if (e == cudaSuccess) e = configure(k_batch_fp64<32>, Lay<double, 32>::bytes * max_warps(32, true));
        break;
    case 64:
        e = configure(k_batch<64>, batch_smem_f32<64>(max_warps(64, false)));
        if (e == cudaSuccess) e = configure(k_batch_fp64<64>, Lay<double, 64>::bytes * max_warps(64, true));
        break;
    }
    return e;
}

cudaError_t launch_batch(int np, const BatchEntry *jobs, int njobs, long long total, unsigned long long *counter,
                         int warps, int num_sms, cudaStream_t st)
{
    switch (np) {
    case 16: return launch_batch_np<16>(jobs, njobs, total, counter, warps, num_sms, st);
    case 32: return launch_batch_np<32>(jobs, njobs, total, counter, warps, num_sms, st);
    case 64: return launch_batch_np<64>(jobs, njobs, total, counter, warps, num_sms, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_batch64(int np, const BatchEntry *jobs, int njobs, int num_sms, cudaStream_t st)
{
    switch (np) {
    case 16: return launch_batch64_np<16>(jobs, njobs, num_sms, st);
    case 32: return launch_batch64_np<32>(jobs, njobs, num_sms, st);
    case 64: return launch_batch64_np<64>(jobs, njobs, num_sms, st);
    }
    return cudaErrorInvalidValue;
}

void fill_params(KParams &P, const fpl_job &jb, int r0, int r1, float amb, float cond_max)
{
    std::memset(&P, 0, sizeof(P));
    P.stack = static_cast<const float2 *>(jb.stack);
    P.nmap = jb.nmap;
    P.phase = static_cast<float2 *>(jb.phase);
    P.tcorr = jb.tcorr;
    P.comp = static_cast<float2 *>(jb.comp);
    P.status = jb.status;
    P.rows = jb.rows;
    P.cols = jb.cols;
    P.nb = jb.nbands;
    P.ny = jb.half_window_y;
    P.nx = jb.half_window_x;
    P.wx = 2 * jb.half_window_x + 1;
    P.K = (2 * jb.half_window_y + 1) * P.wx;
    P.nulong = (P.K + 31) / 32;
    P.plane = (long long)jb.rows * jb.cols;
    P.pix_begin = (long long)r0 * jb.cols;
    P.npix = (long long)(r1 - r0) * jb.cols;
    P.method = jb.method;
    P.semantics = jb.semantics;
    P.mini = jb.mini_stack_count;
    P.bw = jb.band_width;
    P.min_neigh = jb.min_neighbors;
    P.amb = amb;
    P.cond_max = cond_max;
    P.shift = kDefaultShift;
    P.shift_backoff = kDefaultShiftBackoff;
}

}  // namespace fpl

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BatchClass {
    int np = 0;
    int first = 0, count = 0;       // entries [first, first+count) of the device table
    long long total = 0;            // pixels
    int warps = 0;                  // CTA shape
};

// one wave of the mixed-form pieces: its Gamma segments and its solve
// entries per padded depth (16/32/64)
struct MixedWave {
    int seg_first = 0, seg_count = 0;
    long long seg_tiles = 0;
    size_t seg_smem = 0;
    int ent_first[3] = {0, 0, 0}, ent_count[3] = {0, 0, 0};
    long long ent_total[3] = {0, 0, 0};
};

struct fpl_batch {
    fpl_ctx *ctx = nullptr;
    int njobs = 0;
    int nent = 0;                    // counter blocks: FP32 jobs, then mixed pieces
    std::vector<MixedWave> waves;
    fpl::BoxSeg *d_segs = nullptr;   // mixed: Gamma segments of every wave
    fpl::BatchEntry *d_ments = nullptr;   // mixed: solve entries of every wave
    fpl::BatchEntry *d_m64 = nullptr;     // mixed: every piece, by padded depth (FP64 settle)
    int m64_first[3] = {0, 0, 0}, m64_count[3] = {0, 0, 0};
    int mixed_warps[3] = {0, 0, 0};  // warps per CTA of the mixed solve launches (0: the most that fit)
    void *d_rec = nullptr;           // mixed: Gamma records and tile infos of one wave
    std::vector<BatchClass> classes;
    fpl::BatchEntry *d_table = nullptr;
    void *d_scratch = nullptr;       // per-job counters, work counters, FP64 lists
    size_t counter_bytes = 0;        // bytes reset before every run
    std::vector<int> job_of_entry;   // entry -> caller's job index
    long long pixels = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap_stream = nullptr;
};

namespace {

constexpr size_t kJobCounterBytes = 64;   // count, err, slow per job

int batch_enqueue(fpl_batch *b, cudaStream_t st)
{
    fpl_ctx *ctx = b->ctx;
    if (cudaMemsetAsync(b->d_scratch, 0, b->counter_bytes, st) != cudaSuccess) return FPL_ERR_CUDA;
    unsigned long long *work = reinterpret_cast<unsigned long long *>(
        static_cast<char *>(b->d_scratch) + kJobCounterBytes * b->njobs);
    for (size_t c = 0; c < b->classes.size(); ++c) {
        const BatchClass &k = b->classes[c];
        if (fpl::launch_batch(k.np, b->d_table + k.first, k.count, k.total, work + c, k.warps, ctx->num_sms, st) !=
            cudaSuccess)
            return FPL_ERR_CUDA;
    }
    static const int kNP[3] = {16, 32, 64};
    for (const MixedWave &w : b->waves) {
        if (w.seg_count && fpl::launch_gram_batch(b->d_segs + w.seg_first, w.seg_count, w.seg_tiles, w.seg_smem,
                                                  ctx->num_sms, st) != cudaSuccess)
            return FPL_ERR_CUDA;
        for (int c = 0; c < 3; ++c)
            if (w.ent_count[c] && fpl::launch_solve_batch(kNP[c], b->d_ments + w.ent_first[c], w.ent_count[c],
                                                          w.ent_total[c], ctx->num_sms, st,
                                                          b->mixed_warps[c]) != cudaSuccess)
                return FPL_ERR_CUDA;
    }
    for (const BatchClass &k : b->classes)
        if (fpl::launch_batch64(k.np, b->d_table + k.first, k.count, ctx->num_sms, st) != cudaSuccess)
            return FPL_ERR_CUDA;
    for (int c = 0; c < 3; ++c)
        if (b->m64_count[c] &&
            fpl::launch_batch64(kNP[c], b->d_m64 + b->m64_first[c], b->m64_count[c], ctx->num_sms, st) != cudaSuccess)
            return FPL_ERR_CUDA;
    return FPL_OK;
}

}  // namespace

extern "C" {

int fpl_batch_destroy(fpl_batch *b)
{
    return fpl_guard([&]() -> int {
        if (!b) return FPL_OK;
        if (b->ctx) cudaSetDevice(b->ctx->device);
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
        if (b->d_table) cudaFree(b->d_table);
        if (b->d_scratch) cudaFree(b->d_scratch);
        if (b->d_segs) cudaFree(b->d_segs);
        if (b->d_ments) cudaFree(b->d_ments);
        if (b->d_m64) cudaFree(b->d_m64);
        if (b->d_rec) cudaFree(b->d_rec);
        delete b;
        return FPL_OK;
    });
}

int fpl_batch_create(fpl_ctx *ctx, const fpl_job *jobs, int njobs, int flags, fpl_batch **out)
{
    return fpl_guard([&]() -> int {
        if (!ctx || !jobs || !out || njobs <= 0) return FPL_ERR_NULL;
        *out = nullptr;
        for (int j = 0; j < njobs; ++j) {
            int rc = fpl_validate_job(&jobs[j]);
            if (rc) return rc;
            if (jobs[j].memory != FPL_MEM_DEVICE) return FPL_ERR_OPTIONS;
        }
        if (cudaSetDevice(ctx->device) != cudaSuccess) return FPL_ERR_CUDA;
        fpl_batch *b = new fpl_batch();
        b->ctx = ctx;
        b->njobs = njobs;
        auto is_mixed = [&](const fpl_job &jb) {
            return jb.precision == FPL_PREC_MIXED && fpl::gram_box_supported(jb.nbands, jb.half_window_y, jb.half_window_x);
        };
        // FP32 jobs, grouped by padded depth
        std::vector<int> order;
        for (int j = 0; j < njobs; ++j)
            if (!is_mixed(jobs[j])) order.push_back(j);
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int c) { return fpl::pick_np(jobs[a].nbands) < fpl::pick_np(jobs[c].nbands); });
        const int nf = (int)order.size();
        // mixed jobs: row pieces of at most kWavePx pixels, packed into waves
        struct Piece { int job, ra, rb; long long px; };
        const long long kWavePx = 1ll << 20;
        std::vector<Piece> pieces;
        for (int j = 0; j < njobs; ++j) {
            if (!is_mixed(jobs[j])) continue;
            const fpl_job &jb = jobs[j];
            const int r0 = jb.row_begin, r1 = jb.row_end <= 0 ? jb.rows : jb.row_end;
            const int step = (int)std::max<long long>(1, kWavePx / jb.cols);
            for (int ra = r0; ra < r1; ra += step) {
                const int rb = std::min(r1, ra + step);
                pieces.push_back({j, ra, rb, (long long)(rb - ra) * jb.cols});
            }
        }
        const int np_ = (int)pieces.size();
        b->nent = nf + np_;
        long long fb_total = 0;
        for (int j = 0; j < njobs; ++j) {
            const fpl_job &jb = jobs[j];
            const int r1 = jb.row_end <= 0 ? jb.rows : jb.row_end;
            fb_total += (long long)(r1 - jb.row_begin) * jb.cols;
        }
        b->pixels = fb_total;
        // scratch: per-entry counters | work counters (one per class, <= 3) | FP64 lists
        b->counter_bytes = kJobCounterBytes * b->nent + 64;
        const size_t scratch = b->counter_bytes + sizeof(long long) * (size_t)std::max<long long>(fb_total, 1);
        if (cudaMalloc(&b->d_scratch, scratch) != cudaSuccess) { fpl_batch_destroy(b); return FPL_ERR_NOMEM; }
        std::vector<fpl::BatchEntry> table(nf);
        long long fb_off = 0;
        char *cnt_base = static_cast<char *>(b->d_scratch);
        long long *lists = reinterpret_cast<long long *>(cnt_base + b->counter_bytes);
        auto set_counters = [&](fpl::KParams &P, int e) {
            P.fb_count = reinterpret_cast<int *>(cnt_base + kJobCounterBytes * e);
            P.err = reinterpret_cast<unsigned *>(cnt_base + kJobCounterBytes * e + 16);
            P.slow = reinterpret_cast<int *>(cnt_base + kJobCounterBytes * e + 32);
            P.fb_list = lists + fb_off;
            P.fb_cap = (int)std::min<long long>(P.npix, 0x7fffffff);
            fb_off += P.npix;
        };
        for (int e = 0; e < nf; ++e) {
            const int j = order[e];
            const fpl_job &jb = jobs[j];
            const int r0 = jb.row_begin, r1 = jb.row_end <= 0 ? jb.rows : jb.row_end;
            fpl::KParams &P = table[e].P;
            fpl::fill_params(P, jb, r0, r1, ctx->amb_scale, ctx->cond_max);
            P.shift = ctx->shift;
            P.shift_backoff = ctx->shift_backoff;
            set_counters(P, e);
            b->job_of_entry.push_back(j);
        }
        // mixed pieces: parameters, waves, records buffer
        if (np_ > 0) {
            std::vector<fpl::KParams> pp(np_);
            std::vector<int> wave_of(np_);
            std::vector<long long> rec_off(np_), info_off(np_);
            size_t rec_max = 0, info_max = 0;
            {
                long long wpx = 0;
                size_t rec = 0, inf = 0;
                int w = -1;
                for (int i = 0; i < np_; ++i) {
                    const Piece &pc = pieces[i];
                    const fpl_job &jb = jobs[pc.job];
                    if (w < 0 || wpx + pc.px > kWavePx) { ++w; wpx = 0; rec = 0; inf = 0; }
                    wave_of[i] = w;
                    wpx += pc.px;
                    const int cstride = fpl::gram_box_record(jb.nbands);
                    rec_off[i] = (long long)rec;
                    info_off[i] = (long long)inf;
                    rec += (size_t)pc.px * cstride;
                    inf += (size_t)pc.px;
                    rec_max = std::max(rec_max, rec);
                    info_max = std::max(info_max, inf);
                }
                b->waves.resize(w + 1);
            }
            const size_t rec_bytes = (sizeof(float) * rec_max + 255) & ~size_t(255);
            if (cudaMalloc(&b->d_rec, rec_bytes + sizeof(int) * std::max<size_t>(info_max, 1)) != cudaSuccess) {
                fpl_batch_destroy(b);
                return FPL_ERR_NOMEM;
            }
            float *recs = static_cast<float *>(b->d_rec);
            int *infos = reinterpret_cast<int *>(static_cast<char *>(b->d_rec) + rec_bytes);
            for (int i = 0; i < np_; ++i) {
                const Piece &pc = pieces[i];
                const fpl_job &jb = jobs[pc.job];
                fpl::KParams &P = pp[i];
                fpl::fill_params(P, jb, pc.ra, pc.rb, ctx->amb_scale, ctx->cond_max);
                P.shift = ctx->shift;
                P.shift_backoff = ctx->shift_backoff;
                set_counters(P, nf + i);
                P.cbuf = reinterpret_cast<float2 *>(recs + rec_off[i]);
                P.cinfo = infos + info_off[i];
                P.cbase = P.pix_begin;
                P.cstride = fpl::gram_box_record(jb.nbands);
                b->job_of_entry.push_back(pc.job);
            }
            // per wave: Gamma segments, entries by padded depth
            std::vector<fpl::BoxSeg> segs;
            std::vector<fpl::BatchEntry> ments;
            for (size_t w = 0; w < b->waves.size(); ++w) {
                MixedWave &mw = b->waves[w];
                mw.seg_first = (int)segs.size();
                for (int i = 0; i < np_; ++i) {
                    if (wave_of[i] != (int)w) continue;
                    fpl::BoxSeg sg;
                    sg.P = pp[i];
                    sg.tile_offset = mw.seg_tiles;
                    mw.seg_tiles += fpl::gram_box_tiles(pp[i]);
                    mw.seg_smem = std::max(mw.seg_smem, fpl::gram_box_smem(pp[i].nb, pp[i].ny, pp[i].nx));
                    segs.push_back(sg);
                }
                mw.seg_count = (int)segs.size() - mw.seg_first;
                for (int c = 0; c < 3; ++c) {
                    const int npd = 16 << c;
                    mw.ent_first[c] = (int)ments.size();
                    for (int i = 0; i < np_; ++i) {
                        if (wave_of[i] != (int)w || fpl::pick_np(pp[i].nb) != npd) continue;
                        fpl::BatchEntry en;
                        en.P = pp[i];
                        en.px_offset = mw.ent_total[c];
                        mw.ent_total[c] += pp[i].npix;
                        ments.push_back(en);
                    }
                    mw.ent_count[c] = (int)ments.size() - mw.ent_first[c];
                }
            }
            // FP64 settle table: every piece, by padded depth
            std::vector<fpl::BatchEntry> m64;
            for (int c = 0; c < 3; ++c) {
                const int npd = 16 << c;
                b->m64_first[c] = (int)m64.size();
                for (int i = 0; i < np_; ++i) {
                    if (fpl::pick_np(pp[i].nb) != npd) continue;
                    fpl::BatchEntry en;
                    en.P = pp[i];
                    en.px_offset = 0;
                    m64.push_back(en);
                }
                b->m64_count[c] = (int)m64.size() - b->m64_first[c];
                if (b->m64_count[c] && fpl::configure_np(npd) != cudaSuccess) { fpl_batch_destroy(b); return FPL_ERR_CUDA; }
            }
            if (cudaMalloc(&b->d_segs, sizeof(fpl::BoxSeg) * std::max<size_t>(segs.size(), 1)) != cudaSuccess ||
                cudaMalloc(&b->d_ments, sizeof(fpl::BatchEntry) * std::max<size_t>(ments.size(), 1)) != cudaSuccess ||
                cudaMalloc(&b->d_m64, sizeof(fpl::BatchEntry) * std::max<size_t>(m64.size(), 1)) != cudaSuccess) {
                fpl_batch_destroy(b);
                return FPL_ERR_NOMEM;
            }
            if (cudaMemcpy(b->d_segs, segs.data(), sizeof(fpl::BoxSeg) * segs.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(b->d_ments, ments.data(), sizeof(fpl::BatchEntry) * ments.size(), cudaMemcpyHostToDevice) !=
                    cudaSuccess ||
                cudaMemcpy(b->d_m64, m64.data(), sizeof(fpl::BatchEntry) * m64.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
                fpl_batch_destroy(b);
                return FPL_ERR_CUDA;
            }
            // kernel attributes are set before any capture
            for (int c = 0; c < 3; ++c)
                if (fpl::prepare_mixed_batch(16 << c) != cudaSuccess) { fpl_batch_destroy(b); return FPL_ERR_CUDA; }
        }
        // classes and their pixel offsets
        for (int e = 0; e < nf;) {
            BatchClass k;
            k.np = fpl::pick_np(table[e].P.nb);
            k.first = e;
            long long off = 0;
            while (e < nf && fpl::pick_np(table[e].P.nb) == k.np) {
                table[e].px_offset = off;
                off += table[e].P.npix;
                ++e;
            }
            k.count = e - k.first;
            k.total = off;
            k.warps = fpl::max_warps(k.np, false);
            if (fpl::configure_np(k.np) != cudaSuccess) { fpl_batch_destroy(b); return FPL_ERR_CUDA; }
            b->classes.push_back(k);
        }
        if (cudaMalloc(&b->d_table, sizeof(fpl::BatchEntry) * std::max(nf, 1)) != cudaSuccess) {
            fpl_batch_destroy(b);
            return FPL_ERR_NOMEM;
        }
        if (nf && cudaMemcpy(b->d_table, table.data(), sizeof(fpl::BatchEntry) * nf, cudaMemcpyHostToDevice) != cudaSuccess) {
            fpl_batch_destroy(b);
            return FPL_ERR_CUDA;
        }
        if (cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
            fpl_batch_destroy(b);
            return FPL_ERR_CUDA;
        }
        // autotune: warps per CTA per class, timed on the batch itself, cached per key
        if (flags & FPL_BATCH_AUTOTUNE) {
            unsigned long long *d_sum = nullptr;
            if (cudaMalloc(&d_sum, sizeof(unsigned long long)) != cudaSuccess) { fpl_batch_destroy(b); return FPL_ERR_NOMEM; }
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            // one untimed run first: the candidates' times then exclude one-time
            // costs (module loading, kernel attributes, first-touch of buffers)
            if (batch_enqueue(b, b->cap_stream) != FPL_OK || cudaStreamSynchronize(b->cap_stream) != cudaSuccess) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                cudaFree(d_sum);
                fpl_batch_destroy(b);
                return FPL_ERR_CUDA;
            }
            for (BatchClass &k : b->classes) {
                // key: (NP, taps of the first job, mean SHP count of the class / 16)
                unsigned long long shp = 0, px = 0;
                int taps = table[k.first].P.K;
                for (int e = k.first; e < k.first + k.count; ++e) {
                    const fpl::KParams &P = table[e].P;
                    cudaMemsetAsync(d_sum, 0, sizeof(unsigned long long), b->cap_stream);
                    fpl::k_popcount<<<256, 256, 0, b->cap_stream>>>(P.nmap + P.pix_begin * P.nulong,
                                                                     P.npix * P.nulong, d_sum);
                    unsigned long long s = 0;
                    cudaMemcpyAsync(&s, d_sum, sizeof(s), cudaMemcpyDeviceToHost, b->cap_stream);
                    cudaStreamSynchronize(b->cap_stream);
                    shp += s;
                    px += (unsigned long long)P.npix;
                }
                const long long key = ((long long)k.np << 40) | ((long long)taps << 16) | (long long)(px ? shp / px / 16 : 0);
                auto it = ctx->tuned_warps.find(key);
                if (it != ctx->tuned_warps.end()) {
                    k.warps = it->second;
                    continue;
                }
                const int wmax = fpl::max_warps(k.np, false);
                int cands[4] = {std::max(1, wmax / 2), std::max(1, (3 * wmax) / 4), wmax, 0};
                float best = 1e30f;
                int best_w = wmax;
                for (int ci = 0; ci < 3; ++ci) {
                    const int w = cands[ci];
                    if (ci > 0 && w == cands[ci - 1]) continue;
                    k.warps = w;
                    cudaEventRecord(e0, b->cap_stream);
                    if (batch_enqueue(b, b->cap_stream) != FPL_OK) break;
                    cudaEventRecord(e1, b->cap_stream);
                    cudaEventSynchronize(e1);
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (ms < best) { best = ms; best_w = w; }
                }
                k.warps = best_w;
                ctx->tuned_warps[key] = best_w;
            }
            // mixed form: warps per CTA of the solve launches of each padded depth,
            // keyed like the FP32 classes with a bit for the form
            for (int c = 0; c < 3; ++c) {
                if (!b->m64_count[c]) continue;
                const int np = 16 << c;
                unsigned long long shp = 0, px = 0;
                int taps = 0;
                std::vector<fpl::BatchEntry> pcs(b->m64_count[c]);
                cudaMemcpy(pcs.data(), b->d_m64 + b->m64_first[c], sizeof(fpl::BatchEntry) * pcs.size(),
                           cudaMemcpyDeviceToHost);
                for (const fpl::BatchEntry &en : pcs) {
                    const fpl::KParams &P = en.P;
                    taps = std::max(taps, P.K);
                    cudaMemsetAsync(d_sum, 0, sizeof(unsigned long long), b->cap_stream);
                    fpl::k_popcount<<<256, 256, 0, b->cap_stream>>>(P.nmap + P.pix_begin * P.nulong,
                                                                     P.npix * P.nulong, d_sum);
                    unsigned long long sum = 0;
                    cudaMemcpyAsync(&sum, d_sum, sizeof(sum), cudaMemcpyDeviceToHost, b->cap_stream);
                    cudaStreamSynchronize(b->cap_stream);
                    shp += sum;
                    px += (unsigned long long)P.npix;
                }
                const long long key = (1ll << 62) | ((long long)np << 40) | ((long long)taps << 16) |
                                      (long long)(px ? shp / px / 16 : 0);
                auto it = ctx->tuned_warps.find(key);
                if (it != ctx->tuned_warps.end()) {
                    b->mixed_warps[c] = it->second;
                    continue;
                }
                const int wmax = fpl::solve_max_warps(np);
                const int cands[3] = {std::max(1, wmax / 2), std::max(1, (3 * wmax) / 4), wmax};
                float best = 1e30f;
                int best_w = wmax;
                for (int ci = 0; ci < 3; ++ci) {
                    const int w = cands[ci];
                    if (ci > 0 && w == cands[ci - 1]) continue;
                    b->mixed_warps[c] = w;
                    cudaEventRecord(e0, b->cap_stream);
                    if (batch_enqueue(b, b->cap_stream) != FPL_OK) break;
                    cudaEventRecord(e1, b->cap_stream);
                    cudaEventSynchronize(e1);
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (ms < best) { best = ms; best_w = w; }
                }
                b->mixed_warps[c] = best_w;
                ctx->tuned_warps[key] = best_w;
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            cudaFree(d_sum);
            if (cudaStreamSynchronize(b->cap_stream) != cudaSuccess) { fpl_batch_destroy(b); return FPL_ERR_CUDA; }
        }
        if (flags & FPL_BATCH_GRAPH) {
            if (cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                fpl_batch_destroy(b);
                return FPL_ERR_CUDA;
            }
            int rc = batch_enqueue(b, b->cap_stream);
            cudaError_t e = cudaStreamEndCapture(b->cap_stream, &b->graph);
            if (rc || e != cudaSuccess || cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) {
                fpl_batch_destroy(b);
                return rc ? rc : FPL_ERR_CUDA;
            }
        }
        *out = b;
        return FPL_OK;
    });
}

int fpl_batch_run(fpl_batch *b, void *stream)
{
    return fpl_guard([&]() -> int {
        if (!b) return FPL_ERR_NULL;
        if (cudaSetDevice(b->ctx->device) != cudaSuccess) return FPL_ERR_CUDA;
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        if (b->exec) return cudaGraphLaunch(b->exec, st) == cudaSuccess ? FPL_OK : FPL_ERR_CUDA;
        return batch_enqueue(b, st);
    });
}

int fpl_batch_stats(const fpl_batch *b, fpl_stats *out)
{
    return fpl_guard([&]() -> int {
        if (!b || !out) return FPL_ERR_NULL;
        std::vector<int> c(b->counter_bytes / sizeof(int));
        if (cudaMemcpy(c.data(), b->d_scratch, b->counter_bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return FPL_ERR_CUDA;
        std::memset(out, 0, sizeof(*out));
        out->pixels = b->pixels;
        unsigned err = 0;
        for (int e = 0; e < b->nent; ++e) {
            out->fp64_pixels += c[(kJobCounterBytes / sizeof(int)) * e];
            err |= (unsigned)c[(kJobCounterBytes / sizeof(int)) * e + 4];
            out->slow_path_pixels += c[(kJobCounterBytes / sizeof(int)) * e + 8];
        }
        return err ? FPL_ERR_DEVICE_CHECK : FPL_OK;
    });
}

}  // extern "C"
