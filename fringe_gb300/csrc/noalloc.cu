// noalloc.cu -- phase linking that allocates no device memory.
//
// fpl_run_noalloc serves callers that cannot call cudaMalloc: a host
// application whose device memory is owned by another allocator (a memory
// pool or framework that forbids outside allocations), or a long-running
// service that must not allocate after start-up.  Such a caller passes its
// own input and output buffers, and the kernels' scratch -- the list of
// pixels settled by the FP64 pass and its counters -- lives in the
// file-scope array below instead of context buffers.  It runs the plain FP32
// form whatever the job's precision: the mixed form's coherence records
// (3.8 KB per pixel at 30 dates) are far beyond a fixed array.
//
// The array is a fixed-size __device__ variable: every GPU that loads this
// library holds its 4 MiB (plus 256 bytes) until the process exits.  Its
// size bounds one call to FPL_NOALLOC_MAX_PIXELS pixels (row_end - row_begin
// rows times cols); larger jobs are rejected with FPL_ERR_NOALLOC_LIMIT and
// can be split into row ranges, which give identical results because
// windows are clipped to the whole scene.
//
// All calls share the one array and each call leaves its contents behind:
// the counters are cleared on the caller's stream at the start of every
// call, and two calls whose work overlaps on the GPU race on the array.
// A call reports no statistics and no device error flags: the one flag the
// kernels raise (FP64 work list full) cannot be set here, because the list
// holds an entry for every pixel a call may cover.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "ctx.h"
#include "fringe_gb300.h"
#include "guard.h"
#include "kernels.h"
#include "pixel.cuh"

namespace {

constexpr size_t kCounterBytes = 256;   // work-list count, error and slow-path counters

__device__ __align__(256) unsigned char g_noalloc_scratch[kCounterBytes +
                                                          sizeof(long long) * FPL_NOALLOC_MAX_PIXELS];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
int g_num_sms[kMaxDevices] = {};

// With the caller's device current: the device address of the scratch array
// in the current CUDA context (host code cannot use the symbol itself as an
// address).  The address is looked up on every call, not cached: it belongs
// to the context that is current, and a cudaDeviceReset or a caller working
// through its own driver context loads the library's module again, possibly
// at another address.  Once the module is loaded in a context the lookup is
// a table read; the first call in a context loads it.  The SM count is a
// property of the device and is cached.
int noalloc_setup(int dev, unsigned char **addr, int *sms)
{
    if (dev < 0 || dev >= kMaxDevices) return FPL_ERR_UNSUPPORTED;
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return FPL_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_num_sms[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            return FPL_ERR_CUDA;
        g_num_sms[dev] = n;
    }
    *addr = static_cast<unsigned char *>(p);
    *sms = g_num_sms[dev];
    return FPL_OK;
}

}  // namespace

extern "C" int fpl_run_noalloc(const fpl_job *job, void *stream)
{
    return fpl_guard([&]() -> int {
        int rc = fpl_validate_job(job);
        if (rc) return rc;
        if (job->memory != FPL_MEM_DEVICE) return FPL_ERR_OPTIONS;
        const int r0 = job->row_begin, r1 = job->row_end <= 0 ? job->rows : job->row_end;
        const long long npix = (long long)(r1 - r0) * job->cols;
        if (npix > FPL_NOALLOC_MAX_PIXELS) return FPL_ERR_NOALLOC_LIMIT;
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return FPL_ERR_CUDA;
        unsigned char *scratch = nullptr;
        int sms = 0;
        rc = noalloc_setup(dev, &scratch, &sms);
        if (rc) return rc;
        cudaStream_t st = static_cast<cudaStream_t>(stream);

        fpl::KParams P;
        std::memset(&P, 0, sizeof(P));
        P.stack = static_cast<const float2 *>(job->stack);
        P.nmap = job->nmap;
        P.phase = static_cast<float2 *>(job->phase);
        P.tcorr = job->tcorr;
        P.comp = static_cast<float2 *>(job->comp);
        P.status = job->status;
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
        P.npix = npix;
        P.method = job->method;
        P.semantics = job->semantics;
        P.mini = job->mini_stack_count;
        P.bw = job->band_width;
        P.min_neigh = job->min_neighbors;
        P.amb = kDefaultAmbScale;
        P.cond_max = kDefaultCondMax;
        P.shift = kDefaultShift;
        P.shift_backoff = kDefaultShiftBackoff;
        P.fb_count = reinterpret_cast<int *>(scratch);
        P.err = reinterpret_cast<unsigned *>(scratch + 16);
        P.slow = reinterpret_cast<int *>(scratch + 32);
        P.fb_list = reinterpret_cast<long long *>(scratch + kCounterBytes);
        P.fb_cap = FPL_NOALLOC_MAX_PIXELS;
        // the counters must start at zero; the list itself is written before it is read
        if (cudaMemsetAsync(scratch, 0, 64, st) != cudaSuccess) return FPL_ERR_CUDA;
        if (npix == 0) return FPL_OK;
        if (fpl::launch_fp32(P, sms, st) != cudaSuccess) return FPL_ERR_CUDA;
        if (fpl::launch_fp64(P, sms, st) != cudaSuccess) return FPL_ERR_CUDA;
        return FPL_OK;
    });
}
