// serve.cu -- continuous-batching request loop for phase-linking jobs.
//
// fpl_server_submit queues a job whose buffers are in host memory (keep them
// valid, and preferably page-locked, until the job is done).  A scheduler
// thread:
//   * admits queued jobs in arrival order while their device footprint
//     (stack, nmap, outputs and FP64 work list) fits the memory budget, and
//     stages their inputs on a copy stream (stream-ordered allocation);
//   * runs "waves" on a compute stream: every resident job whose inputs
//     have arrived contributes a slice of rows (a fair share of the wave's
//     pixel budget), and the slices of all jobs run as one persistent batch
//     launch per padded depth and form (plain FP32; or, for jobs asking for
//     the mixed-precision form, one tensor-core Gamma launch over the tiles
//     of their slices and one solve launch) plus one FP64 settle launch --
//     jobs that arrive while a wave runs join the next wave;
//   * copies a finished job's outputs back on the copy stream, frees its
//     device memory and wakes its waiters.
// Copies overlap with waves.  Each pixel's result depends only on its own
// job's inputs (windows are clipped to the job's scene), so a job's output
// is the same alone and in any mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "batch.h"
#include "ctx.h"
#include "fringe_gb300.h"
#include "guard.h"
#include "kernels.h"

namespace {

using clk = std::chrono::steady_clock;

double ms_since(clk::time_point t0, clk::time_point t1)
{
    return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

enum JobState { PENDING, STAGING, READY, DRAINING, DONE, FAILED };

struct SJob {
    unsigned long long ticket = 0;
    fpl_job host{}, dev{};
    size_t bytes = 0;
    void *dmem = nullptr;
    int r0 = 0, r1 = 0, next_row = 0, rows_done = 0;
    long long fb_entries = 0;
    JobState state = PENDING;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    clk::time_point t_submit, t_admit, t_first, t_done;
    bool started = false;
    int rc = 0;
};

struct Piece {
    SJob *job;
    int ra, rb;
    int np;
    int mixed;     // 1: mixed-precision form
};

constexpr size_t kPieceCounterBytes = 64;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

struct fpl_server {
    fpl_server_config cfg{};
    int num_sms = 0;
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    bool stop = false;
    unsigned long long next_ticket = 1;
    std::deque<SJob *> pending;
    std::vector<SJob *> active;
    std::map<unsigned long long, SJob *> jobs;
    size_t used = 0;
    cudaStream_t s_copy = nullptr, s_compute = nullptr;
    cudaEvent_t ev_wave = nullptr;
    int max_pieces = 256;
    fpl::BatchEntry *d_table = nullptr, *h_table = nullptr;
    fpl::BoxSeg *d_segs = nullptr, *h_segs = nullptr;   // Gamma segments of a wave's mixed pieces
    void *d_rec = nullptr;                              // their Gamma records and tile infos
    size_t rec_cap = 0;
    void *d_wave = nullptr;
    size_t wave_bytes = 0;
    int fatal = 0;
    long long waves = 0;
};

namespace {

size_t footprint(const fpl_job &j)
{
    const size_t P = (size_t)j.rows * j.cols;
    const int nl = ((2 * j.half_window_y + 1) * (2 * j.half_window_x + 1) + 31) / 32;
    size_t b = 0;
    b += align256(P * j.nbands * 8);   // stack
    b += align256(P * nl * 4);         // nmap
    b += align256(P * j.nbands * 8);   // phase
    b += align256(P * 4);              // tcorr
    b += align256(P * 8);              // comp
    if (j.status) b += align256(P * 4);
    return b;
}

// device copies of the job (pointers inside one allocation)
void carve(SJob *sj)
{
    const fpl_job &j = sj->host;
    const size_t P = (size_t)j.rows * j.cols;
    const int nl = ((2 * j.half_window_y + 1) * (2 * j.half_window_x + 1) + 31) / 32;
    char *p = static_cast<char *>(sj->dmem);
    sj->dev = j;
    sj->dev.memory = FPL_MEM_DEVICE;
    sj->dev.stack = p; p += align256(P * j.nbands * 8);
    sj->dev.nmap = reinterpret_cast<const uint32_t *>(p); p += align256(P * nl * 4);
    sj->dev.phase = p; p += align256(P * j.nbands * 8);
    sj->dev.tcorr = reinterpret_cast<float *>(p); p += align256(P * 4);
    sj->dev.comp = p; p += align256(P * 8);
    sj->dev.status = j.status ? reinterpret_cast<int32_t *>(p) : nullptr;
}

void fail_all(fpl_server *s, int rc)
{
    s->fatal = rc;
    for (SJob *j : s->active) {
        j->state = FAILED;
        j->rc = rc;
    }
    s->active.clear();
    for (SJob *j : s->pending) {
        j->state = FAILED;
        j->rc = rc;
    }
    s->pending.clear();
}

// admit queued jobs that fit the budget (caller holds the lock)
void admit(fpl_server *s)
{
    while (!s->pending.empty()) {
        SJob *j = s->pending.front();
        if (s->used + j->bytes > s->cfg.memory_budget && !s->active.empty()) break;
        if (s->used + j->bytes > s->cfg.memory_budget && s->active.empty() && j->bytes > s->cfg.memory_budget) {
            // larger than the whole budget: refuse it
            s->pending.pop_front();
            j->state = FAILED;
            j->rc = FPL_ERR_NOMEM;
            continue;
        }
        s->pending.pop_front();
        if (cudaMallocAsync(&j->dmem, j->bytes, s->s_copy) != cudaSuccess) {
            j->state = FAILED;
            j->rc = FPL_ERR_NOMEM;
            continue;
        }
        carve(j);
        const size_t P = (size_t)j->host.rows * j->host.cols;
        const int nl = ((2 * j->host.half_window_y + 1) * (2 * j->host.half_window_x + 1) + 31) / 32;
        cudaMemcpyAsync(const_cast<void *>(j->dev.stack), j->host.stack, P * j->host.nbands * 8,
                        cudaMemcpyHostToDevice, s->s_copy);
        cudaMemcpyAsync(const_cast<uint32_t *>(j->dev.nmap), j->host.nmap, P * nl * 4, cudaMemcpyHostToDevice,
                        s->s_copy);
        cudaEventRecord(j->ev_in, s->s_copy);
        j->state = STAGING;
        j->t_admit = clk::now();
        s->used += j->bytes;
        s->active.push_back(j);
    }
}

// one wave over the READY jobs; returns false on a CUDA error
bool run_wave(fpl_server *s, std::vector<Piece> &pieces)
{
    // fair share of the wave's pixels, at least one row per job
    std::vector<SJob *> ready;
    for (SJob *j : s->active)
        if (j->state == READY && j->next_row < j->r1) ready.push_back(j);
    pieces.clear();
    if (ready.empty()) return true;
    const long long budget = s->cfg.wave_pixels;
    const long long share = std::max<long long>(1, budget / (long long)ready.size());
    long long total = 0;
    for (SJob *j : ready) {
        if ((int)pieces.size() >= s->max_pieces) break;
        int rows = (int)std::max<long long>(1, share / j->host.cols);
        const int ra = j->next_row, rb = std::min(j->r1, ra + rows);
        j->next_row = rb;
        if (!j->started) { j->started = true; j->t_first = clk::now(); }
        const int mixed = (j->host.precision == FPL_PREC_MIXED &&
                           fpl::gram_box_supported(j->host.nbands, j->host.half_window_y, j->host.half_window_x))
                              ? 1
                              : 0;
        pieces.push_back({j, ra, rb, fpl::pick_np(j->host.nbands), mixed});
        total += (long long)(rb - ra) * j->host.cols;
    }
    std::stable_sort(pieces.begin(), pieces.end(), [](const Piece &a, const Piece &b) {
        return a.np != b.np ? a.np < b.np : a.mixed < b.mixed;
    });
    // Gamma records of the wave's mixed pieces
    size_t rec_floats = 0, infos = 0;
    for (const Piece &pc : pieces)
        if (pc.mixed) {
            const size_t px = (size_t)(pc.rb - pc.ra) * pc.job->host.cols;
            rec_floats += px * fpl::gram_box_record(pc.job->host.nbands);
            infos += px;
        }
    const size_t rec_bytes = (sizeof(float) * rec_floats + 255) & ~size_t(255);
    if (rec_floats && rec_bytes + sizeof(int) * infos > s->rec_cap) {
        // the previous wave has finished (its event was waited for)
        if (s->d_rec) cudaFree(s->d_rec);
        s->d_rec = nullptr;
        s->rec_cap = 0;
        if (cudaMalloc(&s->d_rec, rec_bytes + sizeof(int) * infos) != cudaSuccess) return false;
        s->rec_cap = rec_bytes + sizeof(int) * infos;
    }
    float *recs = static_cast<float *>(s->d_rec);
    int *rinfo = reinterpret_cast<int *>(static_cast<char *>(s->d_rec) + rec_bytes);
    long long roff = 0, ioff = 0;
    // table (pixel offsets restart in every depth class), counters, work lists
    char *base = static_cast<char *>(s->d_wave);
    long long *lists = reinterpret_cast<long long *>(base + kPieceCounterBytes * s->max_pieces + 64);
    long long loff = 0, coff = 0;
    for (size_t e = 0; e < pieces.size(); ++e) {
        const Piece &pc = pieces[e];
        if (e > 0 && (pieces[e - 1].np != pc.np || pieces[e - 1].mixed != pc.mixed)) coff = 0;
        fpl::KParams &P = s->h_table[e].P;
        fpl::fill_params(P, pc.job->dev, pc.ra, pc.rb, kDefaultAmbScale, kDefaultCondMax);
        P.fb_count = reinterpret_cast<int *>(base + kPieceCounterBytes * e);
        P.err = reinterpret_cast<unsigned *>(base + kPieceCounterBytes * e + 16);
        P.slow = reinterpret_cast<int *>(base + kPieceCounterBytes * e + 32);
        P.fb_list = lists + loff;
        P.fb_cap = (int)P.npix;
        if (pc.mixed) {
            P.cbuf = reinterpret_cast<float2 *>(recs + roff);
            P.cinfo = rinfo + ioff;
            P.cbase = P.pix_begin;
            P.cstride = fpl::gram_box_record(P.nb);
            roff += P.npix * P.cstride;
            ioff += P.npix;
        }
        s->h_table[e].px_offset = coff;
        coff += P.npix;
        loff += P.npix;
    }
    // Gamma segments of the mixed pieces
    int nseg = 0;
    long long tiles = 0;
    size_t gsm = 0;
    for (size_t e = 0; e < pieces.size(); ++e) {
        const fpl::KParams &P = s->h_table[e].P;
        if (!pieces[e].mixed) continue;
        fpl::BoxSeg &sg = s->h_segs[nseg++];
        sg.P = P;
        sg.tile_offset = tiles;
        tiles += fpl::gram_box_tiles(P);
        gsm = std::max(gsm, fpl::gram_box_smem(P.nb, P.ny, P.nx));
    }
    if (nseg &&
        cudaMemcpyAsync(s->d_segs, s->h_segs, sizeof(fpl::BoxSeg) * nseg, cudaMemcpyHostToDevice,
                        s->s_compute) != cudaSuccess)
        return false;
    if (cudaMemcpyAsync(s->d_table, s->h_table, sizeof(fpl::BatchEntry) * pieces.size(), cudaMemcpyHostToDevice,
                        s->s_compute) != cudaSuccess)
        return false;
    if (cudaMemsetAsync(s->d_wave, 0, kPieceCounterBytes * s->max_pieces + 64, s->s_compute) != cudaSuccess)
        return false;
    unsigned long long *work = reinterpret_cast<unsigned long long *>(base + kPieceCounterBytes * s->max_pieces);
    if (nseg && fpl::launch_gram_batch(s->d_segs, nseg, tiles, gsm, s->num_sms, s->s_compute) != cudaSuccess)
        return false;
    size_t e = 0;
    int cls = 0;
    while (e < pieces.size()) {
        const int np = pieces[e].np, mixed = pieces[e].mixed;
        const size_t first = e;
        long long n_px = 0;
        while (e < pieces.size() && pieces[e].np == np && pieces[e].mixed == mixed) n_px += s->h_table[e++].P.npix;
        if (fpl::configure_np(np) != cudaSuccess) return false;
        if (mixed) {
            if (fpl::prepare_mixed_batch(np) != cudaSuccess) return false;
            if (fpl::launch_solve_batch(np, s->d_table + first, (int)(e - first), n_px, s->num_sms, s->s_compute) !=
                cudaSuccess)
                return false;
        } else if (fpl::launch_batch(np, s->d_table + first, (int)(e - first), n_px, work + cls,
                                     fpl::max_warps(np, false), s->num_sms, s->s_compute) != cudaSuccess) {
            return false;
        }
        if (fpl::launch_batch64(np, s->d_table + first, (int)(e - first), s->num_sms, s->s_compute) != cudaSuccess)
            return false;
        ++cls;
    }
    (void)total;
    return cudaEventRecord(s->ev_wave, s->s_compute) == cudaSuccess;
}

void scheduler_loop(fpl_server *s)
{
    cudaSetDevice(s->cfg.device);
    std::vector<Piece> pieces;
    while (true) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->stop && s->pending.empty() && s->active.empty()) break;
            admit(s);
        }
        bool busy = false;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (SJob *j : s->active)
                if (j->state == STAGING && cudaEventQuery(j->ev_in) == cudaSuccess) j->state = READY;
        }
        if (!run_wave(s, pieces)) {
            std::lock_guard<std::mutex> lk(s->mu);
            fail_all(s, FPL_ERR_CUDA);
            s->cv.notify_all();
            continue;
        }
        if (!pieces.empty()) {
            busy = true;
            s->waves++;
            // while the wave runs: admit and stage new arrivals (bounded wait)
            const auto t_wave = clk::now();
            while (cudaEventQuery(s->ev_wave) == cudaErrorNotReady) {
                {
                    std::lock_guard<std::mutex> lk(s->mu);
                    admit(s);
                }
                if (ms_since(t_wave, clk::now()) > 600e3) break;
                std::this_thread::sleep_for(std::chrono::microseconds(50));
            }
            if (cudaEventQuery(s->ev_wave) != cudaSuccess) {
                std::lock_guard<std::mutex> lk(s->mu);
                fail_all(s, FPL_ERR_CUDA);
                s->cv.notify_all();
                continue;
            }
            // jobs whose last rows just finished: copy results back
            std::lock_guard<std::mutex> lk(s->mu);
            for (const Piece &pc : pieces) {
                SJob *j = pc.job;
                j->rows_done += pc.rb - pc.ra;
                if (j->rows_done == j->r1 - j->r0 && j->state == READY) {
                    const fpl_job &h = j->host;
                    const size_t P = (size_t)h.rows * h.cols;
                    const size_t off = (size_t)j->r0 * h.cols, cnt = (size_t)(j->r1 - j->r0) * h.cols;
                    cudaStreamWaitEvent(s->s_copy, s->ev_wave, 0);
                    for (int b = 0; b < h.nbands; ++b)
                        cudaMemcpyAsync(static_cast<char *>(h.phase) + (b * P + off) * 8,
                                        static_cast<char *>(j->dev.phase) + (b * P + off) * 8, cnt * 8,
                                        cudaMemcpyDeviceToHost, s->s_copy);
                    cudaMemcpyAsync(h.tcorr + off, j->dev.tcorr + off, cnt * 4, cudaMemcpyDeviceToHost, s->s_copy);
                    cudaMemcpyAsync(static_cast<char *>(h.comp) + off * 8, static_cast<char *>(j->dev.comp) + off * 8,
                                    cnt * 8, cudaMemcpyDeviceToHost, s->s_copy);
                    if (h.status)
                        cudaMemcpyAsync(h.status + off, j->dev.status + off, cnt * 4, cudaMemcpyDeviceToHost, s->s_copy);
                    cudaEventRecord(j->ev_out, s->s_copy);
                    j->state = DRAINING;
                }
            }
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (size_t k = 0; k < s->active.size();) {
                SJob *j = s->active[k];
                if (j->state == DRAINING && cudaEventQuery(j->ev_out) == cudaSuccess) {
                    cudaFreeAsync(j->dmem, s->s_copy);
                    j->dmem = nullptr;
                    s->used -= j->bytes;
                    j->t_done = clk::now();
                    j->state = DONE;
                    s->active.erase(s->active.begin() + k);
                    s->cv.notify_all();
                    busy = true;
                } else {
                    ++k;
                }
            }
            for (SJob *j : s->active)
                if (j->state == DRAINING || j->state == STAGING) busy = true;
        }
        if (!busy) {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait_for(lk, std::chrono::milliseconds(1));
        }
    }
    cudaStreamSynchronize(s->s_copy);
}

// the scheduler thread: an exception (a host allocation that failed while
// admitting jobs or building a wave) must not end the process, so it fails
// every job with FPL_ERR_HOST, which later submissions also receive, and
// the thread ends
void scheduler(fpl_server *s)
{
    try {
        scheduler_loop(s);
    } catch (...) {
        std::lock_guard<std::mutex> lk(s->mu);
        fail_all(s, FPL_ERR_HOST);
        s->cv.notify_all();
    }
}

}  // namespace

extern "C" {

void fpl_server_config_default(fpl_server_config *c)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->memory_budget = (size_t)80 << 30;   // 80 GB
    c->wave_pixels = 1 << 20;
    c->device = 0;
}

int fpl_server_create(const fpl_server_config *cfg, fpl_server **out)
{
    return fpl_guard([&]() -> int {
        if (!cfg || !out) return FPL_ERR_NULL;
        *out = nullptr;
        if (cfg->wave_pixels <= 0 || cfg->memory_budget == 0) return FPL_ERR_OPTIONS;
        if (cudaSetDevice(cfg->device) != cudaSuccess) return FPL_ERR_CUDA;
        fpl_server *s = new fpl_server();
        s->cfg = *cfg;
        cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, cfg->device);
        bool ok = cudaStreamCreateWithFlags(&s->s_copy, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&s->s_compute, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaEventCreateWithFlags(&s->ev_wave, cudaEventDisableTiming) == cudaSuccess &&
                  cudaMalloc(&s->d_table, sizeof(fpl::BatchEntry) * s->max_pieces) == cudaSuccess &&
                  cudaMallocHost(&s->h_table, sizeof(fpl::BatchEntry) * s->max_pieces) == cudaSuccess &&
                  cudaMalloc(&s->d_segs, sizeof(fpl::BoxSeg) * s->max_pieces) == cudaSuccess &&
                  cudaMallocHost(&s->h_segs, sizeof(fpl::BoxSeg) * s->max_pieces) == cudaSuccess;
        // counters | work counters | work lists (a wave holds at most wave_pixels
        // plus one row per job beyond its share)
        s->wave_bytes = kPieceCounterBytes * s->max_pieces + 64 +
                        sizeof(long long) * (size_t)(cfg->wave_pixels + (long long)s->max_pieces * 65536);
        ok = ok && cudaMalloc(&s->d_wave, s->wave_bytes) == cudaSuccess;
        if (!ok) {
            s->stop = true;
            fpl_server_destroy(s);
            return FPL_ERR_NOMEM;
        }
        try {
            s->th = std::thread(scheduler, s);
        } catch (...) {
            s->stop = true;
            fpl_server_destroy(s);       // no scheduler thread to join
            return FPL_ERR_HOST;
        }
        *out = s;
        return FPL_OK;
    });
}

int fpl_server_submit(fpl_server *s, const fpl_job *job, unsigned long long *ticket)
{
    return fpl_guard([&]() -> int {
        if (!s || !ticket) return FPL_ERR_NULL;
        int rc = fpl_validate_job(job);
        if (rc) return rc;
        if (job->memory != FPL_MEM_HOST) return FPL_ERR_OPTIONS;
        if (job->cols > 65536) return FPL_ERR_UNSUPPORTED;   // a row must fit the wave's work list slack
        SJob *j = new SJob();
        j->host = *job;
        j->bytes = footprint(*job);
        j->r0 = job->row_begin;
        j->r1 = job->row_end <= 0 ? job->rows : job->row_end;
        j->next_row = j->r0;
        j->t_submit = clk::now();
        if (cudaEventCreateWithFlags(&j->ev_in, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&j->ev_out, cudaEventDisableTiming) != cudaSuccess) {
            delete j;
            return FPL_ERR_CUDA;
        }
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->fatal) {
            delete j;
            return s->fatal;
        }
        j->ticket = s->next_ticket++;
        s->jobs[j->ticket] = j;
        s->pending.push_back(j);
        *ticket = j->ticket;
        s->cv.notify_all();
        return FPL_OK;
    });
}

int fpl_server_wait(fpl_server *s, unsigned long long ticket, double timeout_s, fpl_ticket_info *info)
{
    return fpl_guard([&]() -> int {
        if (!s) return FPL_ERR_NULL;
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->jobs.find(ticket);
        if (it == s->jobs.end()) return FPL_ERR_OPTIONS;
        SJob *j = it->second;
        const auto deadline = clk::now() + std::chrono::duration<double>(timeout_s);
        while (j->state != DONE && j->state != FAILED) {
            if (s->cv.wait_until(lk, deadline) == std::cv_status::timeout &&
                j->state != DONE && j->state != FAILED)
                return FPL_ERR_TIMEOUT;
        }
        if (info) {
            info->queue_ms = j->state == DONE ? ms_since(j->t_submit, j->t_admit) : 0.0;
            info->run_ms = j->state == DONE ? ms_since(j->t_admit, j->t_done) : 0.0;
            info->total_ms = j->state == DONE ? ms_since(j->t_submit, j->t_done) : 0.0;
            info->rc = j->rc;
        }
        const int rc = j->state == DONE ? FPL_OK : (j->rc ? j->rc : FPL_ERR_CUDA);
        if (j->dmem) {
            // a job that failed while it held device memory (a finished job
            // has returned it): release it once the server's streams are idle
            cudaStreamSynchronize(s->s_compute);
            cudaStreamSynchronize(s->s_copy);
            cudaFree(j->dmem);
        }
        cudaEventDestroy(j->ev_in);
        cudaEventDestroy(j->ev_out);
        s->jobs.erase(it);
        delete j;
        return rc;
    });
}

int fpl_server_destroy(fpl_server *s)
{
    return fpl_guard([&]() -> int {
        if (!s) return FPL_OK;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
            s->cv.notify_all();
        }
        if (s->th.joinable()) s->th.join();
        cudaSetDevice(s->cfg.device);
        // nothing of the server's may still run when its memory is freed
        if (s->s_compute) cudaStreamSynchronize(s->s_compute);
        if (s->s_copy) cudaStreamSynchronize(s->s_copy);
        for (auto &kv : s->jobs) {
            if (kv.second->ev_in) cudaEventDestroy(kv.second->ev_in);
            if (kv.second->ev_out) cudaEventDestroy(kv.second->ev_out);
            if (kv.second->dmem) cudaFree(kv.second->dmem);     // a job failed while it held memory
            delete kv.second;
        }
        if (s->d_wave) cudaFree(s->d_wave);
        if (s->d_table) cudaFree(s->d_table);
        if (s->h_table) cudaFreeHost(s->h_table);
        if (s->d_segs) cudaFree(s->d_segs);
        if (s->h_segs) cudaFreeHost(s->h_segs);
        if (s->d_rec) cudaFree(s->d_rec);
        if (s->ev_wave) cudaEventDestroy(s->ev_wave);
        if (s->s_copy) cudaStreamDestroy(s->s_copy);
        if (s->s_compute) cudaStreamDestroy(s->s_compute);
        delete s;
        return FPL_OK;
    });
}

}  // extern "C"
