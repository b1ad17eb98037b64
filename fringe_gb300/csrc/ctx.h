// ctx.h -- the library context behind the opaque fpl_ctx handle.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "fringe_gb300.h"

// host-memory runs: row chunks whose copies overlap the compute, and the
// 64-byte counter block of each chunk
constexpr int kRunChunks = 8;
constexpr size_t kCounterBlock = 64;

// default tuning of the FP32 form
constexpr float kDefaultAmbScale = 8.0f;    // FP32 rounding band, in units of n*eps*|A|_F
constexpr float kDefaultCondMax = 1000.0f;  // |C| inverted in FP32 up to this inf-norm condition
constexpr float kDefaultShift = 0.999f;     // inverse-iteration shift, in units of min(1, rho)
constexpr float kDefaultShiftBackoff = 0.97f;   // second shift when M - sigma I is not definite

struct fpl_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t s_in = nullptr, s_out = nullptr;   // copy streams of host-memory runs
    std::vector<cudaEvent_t> chunk_ev;            // 2 per chunk: inputs arrived, chunk computed
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_last = nullptr;   // end of the last run enqueued on this context
    bool last_used = false;
    // staging buffers for host-memory jobs (grown on demand)
    void *d_stack = nullptr, *d_nmap = nullptr, *d_phase = nullptr, *d_tcorr = nullptr,
         *d_comp = nullptr, *d_status = nullptr;
    size_t cap_stack = 0, cap_nmap = 0, cap_phase = 0, cap_tcorr = 0, cap_comp = 0,
           cap_status = 0;
    // scratch: FP64 work list, and d_small = {count, .., err flags}
    void *d_fb_list = nullptr;
    size_t cap_fb_list = 0;
    void *d_small = nullptr;
    // mixed form: packed coherence matrices of one chunk of rows
    void *d_cbuf = nullptr, *d_cinfo = nullptr;
    size_t cap_cbuf = 0, cap_cinfo = 0;
    // nmap: sorted amplitudes, validity and staging of host jobs
    void *d_nm = nullptr;
    size_t cap_nm = 0;
    // host-memory runs: outputs of the FP64-settled pixels, packed for the
    // copy back (device) and received (host)
    void *d_pack = nullptr;
    size_t cap_pack = 0;
    std::vector<float2> h_pack;
    // tuning
    float amb_scale = kDefaultAmbScale;
    float cond_max = kDefaultCondMax;
    float shift = kDefaultShift, shift_backoff = kDefaultShiftBackoff;
    bool force_fp64 = false;
    // optional per-kernel timing: an event pair around every compute launch,
    // tagged with the kernel (enum fpl_kernel_tag)
    bool profile = false;
    std::vector<cudaEvent_t> prof_ev;   // event pool; pair p = events 2p, 2p+1
    std::vector<int> prof_tag;          // tag of pair p
    size_t prof_runs = 0;               // runs enqueued since the last read
    double prof_ms[FPL_KTAG_COUNT] = {};   // per-tag sums of the last read
    fpl_stats stats = {};
    // autotuned warps per CTA of batch launches, keyed by (depth, taps, SHP density)
    std::map<long long, int> tuned_warps;
    std::string last_error;
};

int fpl_validate_job(const fpl_job *job);
// What one fpl_enqueue call enqueues: the FP32 / mixed kernels, the FP64
// settle of the pixels on the work list, and the clearing of the counters
// (which starts a new work list).
enum { ENQ_KERNELS = 1, ENQ_SETTLE = 2, ENQ_RESET = 4, ENQ_ALL = 7 };
// Enqueues one run (rows [row_begin, row_end) of job) on st for device
// buffers; counters: a kCounterBlock-byte block of device memory (NULL: the
// context's first block); count_run: count it as a run for the profiler;
// list_cap: entries of the work list (0: the pixels of the row range; a
// run enqueued as several row ranges with one settle at the end passes the
// pixels of the whole run).
int fpl_enqueue(fpl_ctx *ctx, const fpl_job *job, const void *stack, const uint32_t *nmap,
                void *phase, float *tcorr, void *comp, int32_t *status, cudaStream_t st,
                bool fp64_all, void *counters = nullptr, bool count_run = true, int stages = ENQ_ALL,
                long long list_cap = 0);
