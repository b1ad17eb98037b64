// api.cu -- C ABI of libfringe_gb300.so: contexts and in-memory runs.
//
// fpl_run replaces the OpenMP pixel loop of evd_process
// (src/evd/evd.cpp:512-788; src/phase_link/phase_link.cpp:479-666) for a
// scene held in memory.  The FP32 kernel handles every pixel; pixels whose
// discrete decisions fall inside the FP32 rounding band are queued on the
// device and settled by the FP64 kernel launched right behind it on the same
// stream.  No host round trip separates the two passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fringe_gb300.h"
#include "guard.h"
#include "ctx.h"
#include "kernels.h"
#include "pixel.cuh"

using fpl::KParams;

namespace {

int cuda_fail(fpl_ctx *ctx, cudaError_t e, const char *what)
{
    if (ctx) {
        ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    }
    if (e == cudaErrorMemoryAllocation) return FPL_ERR_NOMEM;
    return FPL_ERR_CUDA;
}

#define FPL_CUDA(ctx, call)                                             \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) return cuda_fail((ctx), _e, #call);      \
    } while (0)

int grow(fpl_ctx *ctx, void **p, size_t *cap, size_t need)
{
    if (*cap >= need) return FPL_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(p, need);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc");
    *cap = need;
    return FPL_OK;
}

// wrapped datum adjustment (python/adjustMiniStacks.py:174-197: the "mul"
// pixel function of a derived VRT band): out[d][p] = phase[d][p] * datum[p]
__global__ void k_adjust_wrapped(const float2 *phase, const float2 *__restrict__ datum, float2 *out,
                                 int ndates, long long npix)
{
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix;
         p += (long long)gridDim.x * blockDim.x) {
        const float2 b = __ldg(datum + p);
        for (int d = 0; d < ndates; ++d) {
            const float2 a = phase[d * npix + p];
            const double re = (double)a.x * b.x - (double)a.y * b.y;
            const double im = (double)a.x * b.y + (double)a.y * b.x;
            out[d * npix + p] = make_float2((float)re, (float)im);
        }
    }
}

}  // namespace

int fpl_validate_job(const fpl_job *job)
{
    if (!job) return FPL_ERR_NULL;
    if (!job->stack || !job->nmap || !job->phase || !job->tcorr || !job->comp) return FPL_ERR_NULL;
    if (job->rows <= 0 || job->cols <= 0 || job->nbands <= 0) return FPL_ERR_OPTIONS;
    if (job->half_window_x < 0 || job->half_window_y < 0) return FPL_ERR_OPTIONS;
    if (job->nbands > FPL_MAX_BANDS) return FPL_ERR_UNSUPPORTED;
    const int K = (2 * job->half_window_y + 1) * (2 * job->half_window_x + 1);
    if ((K + 31) / 32 > FPL_MAX_NULONG) return FPL_ERR_UNSUPPORTED;
    if (job->method < FPL_METHOD_MLE || job->method > FPL_METHOD_STBAS) return FPL_ERR_OPTIONS;
    if (job->semantics != FPL_SEM_EVD && job->semantics != FPL_SEM_PHASE_LINK) return FPL_ERR_OPTIONS;
    if (job->mini_stack_count < 1 || job->mini_stack_count > job->nbands) return FPL_ERR_OPTIONS;
    if (job->method == FPL_METHOD_STBAS) {
        // src/evd/evd.cpp:74-91
        if (job->band_width <= 0 || job->band_width >= job->nbands - 1) return FPL_ERR_OPTIONS;
    }
    if (job->precision != FPL_PREC_FP32 && job->precision != FPL_PREC_MIXED) return FPL_ERR_OPTIONS;
    if (job->memory != FPL_MEM_HOST && job->memory != FPL_MEM_DEVICE) return FPL_ERR_OPTIONS;
    int r0 = job->row_begin, r1 = job->row_end <= 0 ? job->rows : job->row_end;
    if (r0 < 0 || r0 > r1 || r1 > job->rows) return FPL_ERR_OPTIONS;
    return FPL_OK;
}

extern "C" {

const char *fpl_version(void) { return "fringe_gb300 0.1 (sm_103a)"; }

const char *fpl_error_string(int code)
{
    switch (code) {
    case FPL_OK: return "ok";
    case FPL_ERR_OPTIONS: return "invalid options";
    case FPL_ERR_OPEN_STACK: return "cannot open the stack dataset";
    case FPL_ERR_OPEN_WEIGHTS: return "cannot open the weights (nmap) dataset";
    case FPL_ERR_WIDTH: return "width mismatch between stack and weights";
    case FPL_ERR_LENGTH: return "length mismatch between stack and weights";
    case FPL_ERR_NULONG: return "weights band count does not match the window";
    case FPL_ERR_HALFWINDOWX: return "HALFWINDOWX of the weights differs from Nx";
    case FPL_ERR_HALFWINDOWY: return "HALFWINDOWY of the weights differs from Ny";
    case FPL_ERR_DATE: return "a stack band has no Date item in the slc metadata domain";
    case FPL_ERR_OUT_EXISTS_DIR: return "output folder already exists";
    case FPL_ERR_OUT_EXISTS_FILE: return "output folder path exists as a file";
    case FPL_ERR_OUT_MKDIR: return "cannot create the output folder";
    case FPL_ERR_CREATE_SLC: return "cannot create an output SLC";
    case FPL_ERR_CREATE_AUX: return "cannot create tcorr / compressed SLC output";
    case FPL_ERR_READ_STACK: return "error reading the stack";
    case FPL_ERR_READ_WEIGHTS: return "error reading the weights";
    case FPL_ERR_WRITE_SLC: return "error writing an output SLC";
    case FPL_ERR_WRITE_AUX: return "error writing tcorr / compressed SLC";
    case FPL_ERR_CUDA: return "CUDA runtime error";
    case FPL_ERR_NOMEM: return "device memory allocation failed";
    case FPL_ERR_UNSUPPORTED: return "unsupported size (nbands > 64 or window > 1024 taps)";
    case FPL_ERR_DEVICE_CHECK: return "a kernel reported an internal error";
    case FPL_ERR_NULL: return "a required pointer is NULL";
    case FPL_ERR_TIMEOUT: return "timed out waiting for a served job";
    case FPL_ERR_HOST: return "host-side failure (out of host memory, or no thread could be started)";
    case FPL_ERR_NOALLOC_LIMIT: return "job exceeds the FPL_NOALLOC_MAX_PIXELS scratch of fpl_run_noalloc";
    }
    return "unknown error";
}

int fpl_ctx_create(int device, fpl_ctx **out)
{
    return fpl_guard([&]() -> int {
        if (!out) return FPL_ERR_NULL;
        *out = nullptr;
        int ndev = 0;
        cudaError_t e = cudaGetDeviceCount(&ndev);
        if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetDeviceCount");
        if (device < 0 || device >= ndev) return FPL_ERR_OPTIONS;
        e = cudaSetDevice(device);
        if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
        fpl_ctx *ctx = new fpl_ctx();
        ctx->device = device;
        cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
        e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete ctx; return cuda_fail(nullptr, e, "cudaStreamCreate"); }
        cudaEventCreate(&ctx->ev0);
        cudaEventCreate(&ctx->ev1);
        cudaEventCreateWithFlags(&ctx->ev_last, cudaEventDisableTiming);
        e = cudaMalloc(&ctx->d_small, kCounterBlock * kRunChunks);
        if (e != cudaSuccess) { fpl_ctx_destroy(ctx); return cuda_fail(nullptr, e, "cudaMalloc"); }
        *out = ctx;
        return FPL_OK;
    });
}

int fpl_ctx_destroy(fpl_ctx *ctx)
{
    return fpl_guard([&]() -> int {
        if (!ctx) return FPL_OK;
        cudaSetDevice(ctx->device);
        if (ctx->stream) cudaStreamSynchronize(ctx->stream);
        for (cudaEvent_t e : ctx->prof_ev) cudaEventDestroy(e);
        for (cudaEvent_t e : ctx->chunk_ev) cudaEventDestroy(e);
        if (ctx->s_in) cudaStreamDestroy(ctx->s_in);
        if (ctx->s_out) cudaStreamDestroy(ctx->s_out);
        void *bufs[] = {ctx->d_stack, ctx->d_nmap, ctx->d_phase, ctx->d_tcorr, ctx->d_comp,
                        ctx->d_status, ctx->d_fb_list, ctx->d_small, ctx->d_cbuf, ctx->d_cinfo,
                        ctx->d_nm, ctx->d_pack};
        for (void *b : bufs)
            if (b) cudaFree(b);
        if (ctx->ev_last) cudaEventDestroy(ctx->ev_last);
        if (ctx->ev0) cudaEventDestroy(ctx->ev0);
        if (ctx->ev1) cudaEventDestroy(ctx->ev1);
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return FPL_OK;
    });
}

int fpl_last_stats(const fpl_ctx *ctx, fpl_stats *out)
{
    return fpl_guard([&]() -> int {
        if (!ctx || !out) return FPL_ERR_NULL;
        *out = ctx->stats;
        return FPL_OK;
    });
}

}  // extern "C"

static int fpl_enqueue_body(fpl_ctx *ctx, const fpl_job *job, const void *stack, const uint32_t *nmap,
                            void *phase, float *tcorr, void *comp, int32_t *status, cudaStream_t st,
                            bool fp64_all, void *counters, bool count_run, int stages, long long list_cap);

// Enqueues both passes on `st` for device buffers.  Scratch: the context's
// work-list buffer (grown with cudaMalloc when too small) and d_small.
int fpl_enqueue(fpl_ctx *ctx, const fpl_job *job, const void *stack, const uint32_t *nmap,
                void *phase, float *tcorr, void *comp, int32_t *status, cudaStream_t st,
                bool fp64_all, void *counters, bool count_run, int stages, long long list_cap)
{
    if (!counters) counters = ctx->d_small;
    // runs sharing this context share its scratch: a run waits for the
    // previous one, whatever stream it was enqueued on (not while capturing,
    // where the graph orders the work)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    FPL_CUDA(ctx, cudaStreamIsCapturing(st, &cap));
    const bool order = (cap == cudaStreamCaptureStatusNone);
    if (order && ctx->last_used) FPL_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_last, 0));
    int rc_ = fpl_enqueue_body(ctx, job, stack, nmap, phase, tcorr, comp, status, st, fp64_all, counters,
                               count_run, stages, list_cap);
    if (rc_) return rc_;
    if (order) {
        FPL_CUDA(ctx, cudaEventRecord(ctx->ev_last, st));
        ctx->last_used = true;
    }
    return FPL_OK;
}

static int fpl_enqueue_body(fpl_ctx *ctx, const fpl_job *job, const void *stack, const uint32_t *nmap,
                            void *phase, float *tcorr, void *comp, int32_t *status, cudaStream_t st,
                            bool fp64_all, void *counters, bool count_run, int stages, long long list_cap)
{
    const int r0 = job->row_begin, r1 = job->row_end <= 0 ? job->rows : job->row_end;
    int rc = 0;
    KParams P;
    std::memset(&P, 0, sizeof(P));
    P.stack = static_cast<const float2 *>(stack);
    P.nmap = nmap;
    P.phase = static_cast<float2 *>(phase);
    P.tcorr = tcorr;
    P.comp = static_cast<float2 *>(comp);
    P.status = status;
    P.rows = job->rows;
    P.cols = job->cols;
    P.nb = job->nbands;
    P.ny = job->half_window_y;
    P.nx = job->half_window_x;
    P.wx = 2 * job->half_window_x + 1;
    P.K = (2 * job->half_window_y + 1) * P.wx;
    P.nulong = (P.K + 31) / 32;
    P.plane = (long long)job->rows * job->cols;
    P.pix_begin = (long long)r0 * job->cols;
    P.npix = (long long)(r1 - r0) * job->cols;
    P.method = job->method;
    P.semantics = job->semantics;
    P.mini = job->mini_stack_count;
    P.bw = job->band_width;
    P.min_neigh = job->min_neighbors;
    P.amb = ctx->amb_scale;
    P.cond_max = ctx->cond_max;
    P.shift = ctx->shift;
    P.shift_backoff = ctx->shift_backoff;
    int *d_count = reinterpret_cast<int *>(counters);
    unsigned *d_err = reinterpret_cast<unsigned *>(static_cast<char *>(counters) + 16);
    P.fb_count = d_count;
    P.err = d_err;
    P.slow = reinterpret_cast<int *>(static_cast<char *>(counters) + 32);
    // work list: at most one entry per pixel of the range (or of the run)
    const long long cap = list_cap > 0 ? list_cap : P.npix;
    size_t need = sizeof(long long) * (size_t)(cap > 0 ? cap : 1);
    rc = grow(ctx, &ctx->d_fb_list, &ctx->cap_fb_list, need);
    if (rc) return rc;
    P.fb_list = static_cast<long long *>(ctx->d_fb_list);
    P.fb_cap = (int)(cap < 0x7fffffff ? cap : 0x7fffffff);
    if (stages & ENQ_RESET) FPL_CUDA(ctx, cudaMemsetAsync(counters, 0, kCounterBlock, st));
    if (P.npix == 0) return FPL_OK;
    if (fp64_all) {
        if (stages & ENQ_KERNELS) {
            KParams Q = P;
            Q.fb_list = nullptr;
            FPL_CUDA(ctx, fpl::launch_fp64(Q, ctx->num_sms, st));
        }
        return FPL_OK;
    }
    // optional per-kernel event pairs (fpl_ctx_set_profiling)
    auto timed = [&](int tag, auto &&launch) -> cudaError_t {
        if (!ctx->profile) return launch();
        const size_t p = ctx->prof_tag.size();
        while (ctx->prof_ev.size() < 2 * (p + 1)) {
            cudaEvent_t e;
            cudaError_t ce = cudaEventCreate(&e);
            if (ce != cudaSuccess) return ce;
            ctx->prof_ev.push_back(e);
        }
        cudaError_t ce = cudaEventRecord(ctx->prof_ev[2 * p], st);
        if (ce != cudaSuccess) return ce;
        if ((ce = launch()) != cudaSuccess) return ce;
        if ((ce = cudaEventRecord(ctx->prof_ev[2 * p + 1], st)) != cudaSuccess) return ce;
        ctx->prof_tag.push_back(tag);
        return cudaSuccess;
    };
    if (ctx->profile && count_run) ctx->prof_runs++;
    const bool mixed = job->precision == FPL_PREC_MIXED && fpl::gram_box_supported(P.nb, P.ny, P.nx);
    if (!(stages & ENQ_KERNELS)) {
        // settle only
    } else if (mixed) {
        // tensor-core Gamma records, then eigen-solves, chunk by chunk of
        // rows so the records stay within a bounded buffer
        const int rec = fpl::gram_box_record(P.nb);
        const long long chunk_px_max = std::max<long long>(P.cols, (1ll << 20));
        const int rows_per_chunk = (int)std::max<long long>(1, chunk_px_max / P.cols);
        const long long chunk_px = (long long)std::min(rows_per_chunk, r1 - r0) * P.cols;
        if ((rc = grow(ctx, &ctx->d_cbuf, &ctx->cap_cbuf, sizeof(float) * (size_t)rec * chunk_px))) return rc;
        if ((rc = grow(ctx, &ctx->d_cinfo, &ctx->cap_cinfo, sizeof(int) * (size_t)chunk_px))) return rc;
        for (int ra = r0; ra < r1; ra += rows_per_chunk) {
            const int rb = std::min(r1, ra + rows_per_chunk);
            KParams Q = P;
            Q.pix_begin = (long long)ra * P.cols;
            Q.npix = (long long)(rb - ra) * P.cols;
            Q.cbuf = static_cast<float2 *>(ctx->d_cbuf);
            Q.cinfo = static_cast<int *>(ctx->d_cinfo);
            Q.cbase = Q.pix_begin;
            Q.cstride = rec;
            FPL_CUDA(ctx, timed(FPL_KTAG_GRAM, [&] { return fpl::launch_gram_box(Q, ctx->num_sms, st); }));
            FPL_CUDA(ctx, timed(FPL_KTAG_SOLVE, [&] { return fpl::launch_solve(Q, ctx->num_sms, st); }));
        }
    } else {
        FPL_CUDA(ctx, timed(FPL_KTAG_FP32, [&] { return fpl::launch_fp32(P, ctx->num_sms, st); }));
    }
    if (stages & ENQ_SETTLE)
        FPL_CUDA(ctx, timed(FPL_KTAG_FP64, [&] { return fpl::launch_fp64(P, ctx->num_sms, st); }));
    return FPL_OK;
}

// Outputs of the pixels on a run's FP64 work list, packed (nb + 3 complex
// slots per pixel: the phases, the compressed SLC, {tcorr, status bits},
// {pixel index low, high bits}) for one copy back to the host.
__global__ void k_pack_settled(const long long *__restrict__ list, const int *__restrict__ count, int cap,
                               const float2 *__restrict__ phase, const float *__restrict__ tcorr,
                               const float2 *__restrict__ comp, const int32_t *__restrict__ status,
                               long long plane, int nb, float2 *__restrict__ out)
{
    const int n = min(*count, cap);
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < (long long)n * (nb + 3);
         k += (long long)gridDim.x * blockDim.x) {
        const long long e = k / (nb + 3);
        const int slot = (int)(k - e * (nb + 3));
        const long long pp = list[e];
        float2 v;
        if (slot < nb) v = phase[slot * plane + pp];
        else if (slot == nb) v = comp[pp];
        else if (slot == nb + 1) v = make_float2(tcorr[pp], __int_as_float(status ? status[pp] : 0));
        else v = make_float2(__int_as_float((int)(pp & 0xffffffffll)), __int_as_float((int)(pp >> 32)));
        out[k] = v;
    }
}

extern "C" {

int fpl_adjust_wrapped(fpl_ctx *ctx, const void *phase, const void *datum, void *out,
                       int ndates, long long npix, void *stream)
{
    return fpl_guard([&]() -> int {
        if (!ctx || !phase || !datum || !out) return FPL_ERR_NULL;
        if (ndates < 0 || npix < 0) return FPL_ERR_OPTIONS;
        if (ndates == 0 || npix == 0) return FPL_OK;
        FPL_CUDA(ctx, cudaSetDevice(ctx->device));
        long long blocks = std::min<long long>((npix + 255) / 256, (long long)ctx->num_sms * 8);
        k_adjust_wrapped<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const float2 *>(phase), static_cast<const float2 *>(datum),
            static_cast<float2 *>(out), ndates, npix);
        FPL_CUDA(ctx, cudaGetLastError());
        return FPL_OK;
    });
}

int fpl_run_async(fpl_ctx *ctx, const fpl_job *job, void *stream)
{
    return fpl_guard([&]() -> int {
        if (!ctx) return FPL_ERR_NULL;
        int rc = fpl_validate_job(job);
        if (rc) return rc;
        if (job->memory != FPL_MEM_DEVICE) return FPL_ERR_OPTIONS;
        FPL_CUDA(ctx, cudaSetDevice(ctx->device));
        // the stream is used as given: NULL is the legacy default stream
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        return fpl_enqueue(ctx, job, job->stack, job->nmap, job->phase, job->tcorr, job->comp,
                           job->status, st, ctx->force_fp64, ctx->d_small, true);
    });
}

// host threads that put the FP64-settled pixels in place after a host-memory run
constexpr int kScatterThreads = 8;

// Host-memory jobs run in row chunks so that copies overlap the compute:
// chunk c's stack rows (with the window apron and the rows of its first and
// last 8-row tiles) and nmap rows go up on a copy stream, the chunk is
// computed on the context's stream once they have arrived, and its outputs
// come back on a third stream while the next chunk computes.  Each chunk has
// its own block of counters so the statistics add up over the run.
int fpl_run(fpl_ctx *ctx, const fpl_job *job)
{
    return fpl_guard([&]() -> int {
        if (!ctx) return FPL_ERR_NULL;
        int rc = fpl_validate_job(job);
        if (rc) return rc;
        auto t0 = std::chrono::steady_clock::now();
        FPL_CUDA(ctx, cudaSetDevice(ctx->device));
        cudaStream_t st = ctx->stream;
        const int rows = job->rows, cols = job->cols, nb = job->nbands, ny = job->half_window_y;
        const size_t plane = (size_t)rows * cols;
        const int nulong = ((2 * job->half_window_y + 1) * (2 * job->half_window_x + 1) + 31) / 32;
        const size_t b_stack = plane * nb * 8, b_nmap = plane * nulong * 4;
        const size_t b_tc = plane * 4, b_comp = plane * 8, b_st = plane * 4;
        const int r0 = job->row_begin, r1 = job->row_end <= 0 ? rows : job->row_end;
        int nchunks = 1;
        if (job->memory == FPL_MEM_DEVICE) {
            FPL_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
            rc = fpl_enqueue(ctx, job, job->stack, job->nmap, job->phase, job->tcorr, job->comp, job->status, st,
                             ctx->force_fp64, ctx->d_small, true);
            if (rc) return rc;
            FPL_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
        } else {
            if ((rc = grow(ctx, &ctx->d_stack, &ctx->cap_stack, b_stack))) return rc;
            if ((rc = grow(ctx, &ctx->d_nmap, &ctx->cap_nmap, b_nmap))) return rc;
            if ((rc = grow(ctx, &ctx->d_phase, &ctx->cap_phase, b_stack))) return rc;
            if ((rc = grow(ctx, &ctx->d_tcorr, &ctx->cap_tcorr, b_tc))) return rc;
            if ((rc = grow(ctx, &ctx->d_comp, &ctx->cap_comp, b_comp))) return rc;
            if (job->status && (rc = grow(ctx, &ctx->d_status, &ctx->cap_status, b_st))) return rc;
            if (!ctx->s_in) FPL_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->s_in, cudaStreamNonBlocking));
            if (!ctx->s_out) FPL_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->s_out, cudaStreamNonBlocking));
            while (ctx->chunk_ev.size() < 2 * (size_t)kRunChunks) {
                cudaEvent_t e;
                FPL_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
                ctx->chunk_ev.push_back(e);
            }
            char *d_stack = static_cast<char *>(ctx->d_stack);
            char *d_phase = static_cast<char *>(ctx->d_phase);
            char *d_comp = static_cast<char *>(ctx->d_comp);
            uint32_t *d_nmap = static_cast<uint32_t *>(ctx->d_nmap);
            float *d_tcorr = static_cast<float *>(ctx->d_tcorr);
            int32_t *d_status = job->status ? static_cast<int32_t *>(ctx->d_status) : nullptr;
            const char *h_stack = static_cast<const char *>(job->stack);
            // chunk c computes rows [cb[c], cb[c+1]).  The first chunk's upload
            // and the last chunk's download overlap no compute, so those chunks
            // are the smallest (row shares 1,2,3,..,3,2,1, multiples of 8
            // rows); short ranges are cut into equal chunks of >= 8 rows.
            int cb[kRunChunks + 1];
            {
                static_assert(kRunChunks == 8, "chunk weights");
                const int wsum[kRunChunks + 1] = {0, 1, 3, 6, 9, 12, 15, 17, 18};
                const int span = r1 - r0;
                cb[0] = r0;
                nchunks = 0;
                if (span >= 8 * 18) {
                    for (int c = 1; c <= kRunChunks; ++c)
                        cb[c] = (c == kRunChunks) ? r1 : r0 + (int)((long long)span * wsum[c] / 18) / 8 * 8;
                    nchunks = kRunChunks;
                } else {
                    int step = (span + kRunChunks - 1) / kRunChunks;
                    step = std::max(8, (step + 7) & ~7);
                    for (int a = r0; a < r1; a += step) cb[++nchunks] = std::min(r1, a + step);
                }
                nchunks = std::max(nchunks, 1);
                if (span <= 0) cb[1] = r1;
            }
            int copied = std::max(0, r0 / 8 * 8 - ny);     // first stack row on the device
            // One work list for the whole run: the chunks append to it and its
            // FP64 settle runs once, after the last chunk (a settle per chunk
            // costs a round of the slow FP64 pixels each time); the settled
            // pixels' outputs then come back packed and are put in place here.
            const long long run_px = (long long)(r1 - r0) * cols;
            FPL_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
            bool first = true;                  // the first chunk clears the counters (starts the list)
            for (int c = 0; c < nchunks; ++c) {
                const int a = cb[c], b = cb[c + 1];
                if (b <= a) continue;
                // stack rows every computed pixel's window (and the chunk's tiles) read
                const int need = std::min(rows, (b + 7) / 8 * 8 + ny);
                if (need > copied) {
                    const size_t off = (size_t)copied * cols * 8;
                    FPL_CUDA(ctx, cudaMemcpy2DAsync(d_stack + off, plane * 8, h_stack + off, plane * 8,
                                                    (size_t)(need - copied) * cols * 8, nb, cudaMemcpyHostToDevice,
                                                    ctx->s_in));
                    copied = need;
                }
                FPL_CUDA(ctx, cudaMemcpyAsync(d_nmap + (size_t)a * cols * nulong, job->nmap + (size_t)a * cols * nulong,
                                              (size_t)(b - a) * cols * nulong * 4, cudaMemcpyHostToDevice, ctx->s_in));
                cudaEvent_t ev_in = ctx->chunk_ev[2 * c], ev_done = ctx->chunk_ev[2 * c + 1];
                FPL_CUDA(ctx, cudaEventRecord(ev_in, ctx->s_in));
                FPL_CUDA(ctx, cudaStreamWaitEvent(st, ev_in, 0));
                fpl_job cj = *job;
                cj.row_begin = a;
                cj.row_end = b;
                rc = fpl_enqueue(ctx, &cj, d_stack, d_nmap, d_phase, d_tcorr, d_comp, d_status, st, ctx->force_fp64,
                                 ctx->d_small, first, ENQ_KERNELS | (first ? ENQ_RESET : 0), run_px);
                if (rc) return rc;
                first = false;
                FPL_CUDA(ctx, cudaEventRecord(ev_done, st));
                FPL_CUDA(ctx, cudaStreamWaitEvent(ctx->s_out, ev_done, 0));
                const size_t off = (size_t)a * cols, cnt = (size_t)(b - a) * cols;
                FPL_CUDA(ctx, cudaMemcpy2DAsync(static_cast<char *>(job->phase) + off * 8, plane * 8, d_phase + off * 8,
                                                plane * 8, cnt * 8, nb, cudaMemcpyDeviceToHost, ctx->s_out));
                FPL_CUDA(ctx, cudaMemcpyAsync(job->tcorr + off, d_tcorr + off, cnt * 4, cudaMemcpyDeviceToHost,
                                              ctx->s_out));
                FPL_CUDA(ctx, cudaMemcpyAsync(static_cast<char *>(job->comp) + off * 8, d_comp + off * 8, cnt * 8,
                                              cudaMemcpyDeviceToHost, ctx->s_out));
                if (job->status)
                    FPL_CUDA(ctx, cudaMemcpyAsync(job->status + off, d_status + off, cnt * 4, cudaMemcpyDeviceToHost,
                                                  ctx->s_out));
            }
            // the FP64 settle of every chunk's list, on the whole range (an empty
            // range only clears the counters)
            rc = fpl_enqueue(ctx, job, d_stack, d_nmap, d_phase, d_tcorr, d_comp, d_status, st, ctx->force_fp64,
                             ctx->d_small, false, first ? ENQ_RESET : ENQ_SETTLE, run_px);
            if (rc) return rc;
            FPL_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
            int head[16];
            FPL_CUDA(ctx, cudaMemcpyAsync(head, ctx->d_small, kCounterBlock, cudaMemcpyDeviceToHost, st));
            FPL_CUDA(ctx, cudaStreamSynchronize(st));
            const long long nset = std::min<long long>(head[0], run_px);
            if (nset > 0 && !ctx->force_fp64) {
                const size_t slots = (size_t)nset * (nb + 3);
                if ((rc = grow(ctx, &ctx->d_pack, &ctx->cap_pack, slots * sizeof(float2)))) return rc;
                const unsigned blocks = (unsigned)std::min<size_t>((slots + 255) / 256, (size_t)ctx->num_sms * 8);
                k_pack_settled<<<blocks, 256, 0, st>>>(static_cast<const long long *>(ctx->d_fb_list),
                                                       static_cast<const int *>(ctx->d_small), (int)nset,
                                                       reinterpret_cast<const float2 *>(d_phase), d_tcorr,
                                                       reinterpret_cast<const float2 *>(d_comp), d_status, (long long)plane,
                                                       nb, static_cast<float2 *>(ctx->d_pack));
                FPL_CUDA(ctx, cudaGetLastError());
                ctx->h_pack.resize(slots);
                FPL_CUDA(ctx, cudaMemcpyAsync(ctx->h_pack.data(), ctx->d_pack, slots * sizeof(float2),
                                              cudaMemcpyDeviceToHost, st));
                FPL_CUDA(ctx, cudaStreamSynchronize(st));
            }
            // every chunk's outputs are on the host before the settled pixels
            // are put in place over them
            FPL_CUDA(ctx, cudaStreamSynchronize(ctx->s_out));
            if (nset > 0 && !ctx->force_fp64) {
                // each settled pixel writes one value into each of nb planes far
                // apart, so the loop waits on cache misses: split it over host
                // threads (pixels appear once in the list, so the ranges write
                // disjoint places)
                float2 *h_phase = static_cast<float2 *>(job->phase), *h_comp = static_cast<float2 *>(job->comp);
                const float2 *pack = ctx->h_pack.data();
                auto put = [&](long long e0, long long e1) {
                    for (long long e = e0; e < e1; ++e) {
                        const float2 *v = pack + (size_t)e * (nb + 3);
                        uint32_t lo, hi;
                        int32_t stv;
                        std::memcpy(&lo, &v[nb + 2].x, 4);
                        std::memcpy(&hi, &v[nb + 2].y, 4);
                        std::memcpy(&stv, &v[nb + 1].y, 4);
                        const long long pp = (long long)(((uint64_t)hi << 32) | lo);
                        for (int b = 0; b < nb; ++b) h_phase[(size_t)b * plane + pp] = v[b];
                        h_comp[pp] = v[nb];
                        job->tcorr[pp] = v[nb + 1].x;
                        if (job->status) job->status[pp] = stv;
                    }
                };
                const long long per_thread = 512;
                const int nt = (int)std::max<long long>(
                    1, std::min<long long>({(long long)kScatterThreads, (long long)std::thread::hardware_concurrency(),
                                            (nset + per_thread - 1) / per_thread}));
                if (nt <= 1) {
                    put(0, nset);
                } else {
                    std::vector<std::thread> pool;
                    pool.reserve(nt - 1);           // only starting a thread can throw below
                    const long long step = (nset + nt - 1) / nt;
                    for (int t = 1; t < nt; ++t) {
                        const long long e0 = std::min(nset, t * step), e1 = std::min(nset, (t + 1) * step);
                        try {
                            pool.emplace_back(put, e0, e1);
                        } catch (...) {
                            put(e0, e1);            // no thread: this one takes the range
                        }
                    }
                    put(0, std::min(nset, step));
                    for (std::thread &th : pool) th.join();
                }
            }
        }
        int small[16];
        FPL_CUDA(ctx, cudaMemcpyAsync(small, ctx->d_small, kCounterBlock, cudaMemcpyDeviceToHost, st));
        FPL_CUDA(ctx, cudaStreamSynchronize(st));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        const long long fp64 = small[0], slow = small[8];
        const unsigned err = static_cast<unsigned>(small[4]);
        ctx->stats.pixels = (long long)(r1 - r0) * cols;
        ctx->stats.fp64_pixels = ctx->force_fp64 ? ctx->stats.pixels : fp64;
        ctx->stats.mixed_fp64_inverse = 0;
        ctx->stats.slow_path_pixels = slow;
        ctx->stats.kernel_ms = ms;
        ctx->stats.total_ms =
            std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (err) {
            ctx->last_error = "device error flags " + std::to_string(err);
            return FPL_ERR_DEVICE_CHECK;
        }
        return FPL_OK;
    });
}

// test hooks: width of the FP32 ambiguity band, and FP64 for every pixel
int fpl_ctx_set_tuning(fpl_ctx *ctx, float amb_scale, int force_fp64)
{
    return fpl_guard([&]() -> int {
        if (!ctx) return FPL_ERR_NULL;
        if (amb_scale >= 0.f) ctx->amb_scale = amb_scale;
        ctx->force_fp64 = force_fp64 != 0;
        return FPL_OK;
    });
}

int fpl_ctx_set_shift(fpl_ctx *ctx, float shift, float backoff)
{
    return fpl_guard([&]() -> int {
        if (!ctx) return FPL_ERR_NULL;
        if (!(shift > 0.f) || !(backoff > 0.f)) return FPL_ERR_OPTIONS;
        ctx->shift = shift;
        ctx->shift_backoff = backoff;
        return FPL_OK;
    });
}

const char *fpl_ctx_last_error(const fpl_ctx *ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int fpl_ctx_set_profiling(fpl_ctx *ctx, int on)
{
    return fpl_guard([&]() -> int {
        if (!ctx) return FPL_ERR_NULL;
        ctx->profile = on != 0;
        ctx->prof_tag.clear();
        ctx->prof_runs = 0;
        return FPL_OK;
    });
}

int fpl_ctx_profile(fpl_ctx *ctx, double *fp32_ms, double *fp64_ms, int *runs)
{
    return fpl_guard([&]() -> int {
        if (!ctx) return FPL_ERR_NULL;
        double ms[FPL_KTAG_COUNT] = {};
        for (size_t p = 0; p < ctx->prof_tag.size(); ++p) {
            FPL_CUDA(ctx, cudaEventSynchronize(ctx->prof_ev[2 * p + 1]));
            float x = 0.f;
            FPL_CUDA(ctx, cudaEventElapsedTime(&x, ctx->prof_ev[2 * p], ctx->prof_ev[2 * p + 1]));
            ms[ctx->prof_tag[p]] += x;
        }
        for (int t = 0; t < FPL_KTAG_COUNT; ++t) ctx->prof_ms[t] = ms[t];
        if (fp32_ms) *fp32_ms = ms[FPL_KTAG_FP32] + ms[FPL_KTAG_GRAM] + ms[FPL_KTAG_SOLVE];
        if (fp64_ms) *fp64_ms = ms[FPL_KTAG_FP64];
        if (runs) *runs = (int)ctx->prof_runs;
        ctx->prof_tag.clear();
        ctx->prof_runs = 0;
        return FPL_OK;
    });
}

int fpl_ctx_profile_kernels(const fpl_ctx *ctx, double *ms, int count)
{
    return fpl_guard([&]() -> int {
        if (!ctx || !ms) return FPL_ERR_NULL;
        for (int t = 0; t < count && t < FPL_KTAG_COUNT; ++t) ms[t] = ctx->prof_ms[t];
        return FPL_OK;
    });
}

}  // extern "C"
