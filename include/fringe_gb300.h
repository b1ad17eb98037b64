/*
 * fringe_gb300.h -- C ABI of the GB300 phase-linking library
 * (libfringe_gb300.so).
 *
 * The library replaces the per-pixel phase-linking loop of FRInGE's evd and
 * phase_link modules with CUDA kernels for sm_103a.  Signatures use only
 * plain C types and pointers; no C++ exceptions cross this boundary.
 *
 * Data layouts are the reference's in-memory layouts:
 *   stack  complex64 (interleaved float re,im), band-planar [nbands][rows][cols]
 *          -- src/evd/evd.cpp:195 (arma::cx_fmat cpxdata(cols*rows, nbands))
 *   nmap   uint32 [rows][cols][nulong], nulong = ceil((2Ny+1)(2Nx+1)/32),
 *          bit layout of include/fringe/ulongmask.hpp:55-94
 *          -- src/evd/evd.cpp:197 (arma::Mat<uint> wts(nulong, pixels))
 *   phase  complex64, band-planar [nbands][rows][cols] (evddata, evd.cpp:196)
 *   tcorr  float32 [rows][cols]   (corr, evd.cpp:198)
 *   comp   complex64 [rows][cols] (comp, evd.cpp:199)
 *
 * Return codes: 0 on success; the reference's module codes 101-121 where the
 * same condition applies (src/evd/evd.cpp:54-121,157-165,213-261,278-355,
 * 467-478,492-503,800-856); device-side failures use codes >= 200.
 */
#ifndef FRINGE_GB300_H
#define FRINGE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- enums -------------------------------------------------------------- */
enum fpl_method {            /* evdOptions::method, src/evd/evd.hpp:42 */
    FPL_METHOD_MLE = 0,
    FPL_METHOD_EVD = 1,
    FPL_METHOD_STBAS = 2
};

enum fpl_semantics {         /* which reference module's loop is mirrored */
    FPL_SEM_EVD = 0,         /* src/evd/evd.cpp:512-788         */
    FPL_SEM_PHASE_LINK = 1   /* src/phase_link/phase_link.cpp:479-666 */
};

enum fpl_precision {
    FPL_PREC_FP32 = 0,       /* plain FP32 form (FP64 only to settle ambiguous decisions) */
    FPL_PREC_MIXED = 1       /* BF16 split-precision tensor-core coherence matrix */
};

enum fpl_memory {
    FPL_MEM_HOST = 0,        /* pointers are host memory; the call stages them */
    FPL_MEM_DEVICE = 1       /* pointers are device memory of the context's GPU */
};

/* per-pixel status values written to fpl_job::status (optional output) */
enum fpl_pixel_status {
    FPL_PX_OK = 0,
    FPL_PX_SKIPPED_CENTRE = 1,    /* centre bit clear, evd.cpp:517 */
    FPL_PX_TOO_FEW = 2,           /* npix < 2 / minNeighbors, evd.cpp:566 */
    FPL_PX_EVD_FALLBACK = 3       /* phase_link: MLE not possible, EVD used */
    /* negative values: the reference's tcorr codes -1 .. -7 */
};

/* return codes (device side; module codes 101-121 follow the reference) */
#define FPL_OK                 0
#define FPL_ERR_OPTIONS        101   /* bad options (evd.cpp:78-91 uses 101) */
#define FPL_ERR_OPEN_STACK     102
#define FPL_ERR_OPEN_WEIGHTS   105
#define FPL_ERR_WIDTH          106
#define FPL_ERR_LENGTH         107
#define FPL_ERR_NULONG         108
#define FPL_ERR_HALFWINDOWX    109
#define FPL_ERR_HALFWINDOWY    110
#define FPL_ERR_DATE           112
#define FPL_ERR_OUT_EXISTS_DIR 113
#define FPL_ERR_OUT_EXISTS_FILE 114
#define FPL_ERR_OUT_MKDIR      115
#define FPL_ERR_CREATE_SLC     116
#define FPL_ERR_CREATE_AUX     117
#define FPL_ERR_READ_STACK     118
#define FPL_ERR_READ_WEIGHTS   119
#define FPL_ERR_WRITE_SLC      120
#define FPL_ERR_WRITE_AUX      121
#define FPL_ERR_CUDA           201   /* a CUDA runtime call failed */
#define FPL_ERR_NOMEM          202   /* device allocation failed */
#define FPL_ERR_UNSUPPORTED    203   /* nbands > 64 or window > 1024 taps */
#define FPL_ERR_DEVICE_CHECK   204   /* a kernel reported an internal error */
#define FPL_ERR_NULL           205   /* a required pointer is NULL */
#define FPL_ERR_NOALLOC_LIMIT  206   /* job larger than fpl_run_noalloc's scratch */
#define FPL_ERR_TIMEOUT        207   /* fpl_server_wait gave up */
#define FPL_ERR_HOST           208   /* host-side failure (host memory, threads) */

#define FPL_MAX_BANDS 64
#define FPL_MAX_NULONG 32

typedef struct fpl_ctx fpl_ctx;

/* ---- in-memory job -------------------------------------------------------
 * One phase-linking pass over a scene held in memory: the body of the
 * reference's per-block loop (src/evd/evd.cpp:512-788 and
 * src/phase_link/phase_link.cpp:479-666) for every pixel of rows
 * [row_begin, row_end) (row_end <= 0 means "to the last row").  Windows are
 * clipped to the scene exactly as the reference's block logic makes them
 * (evd.cpp:419-443,530-534), so results do not depend on blocking.        */
typedef struct {
    int rows, cols, nbands;
    int half_window_y;       /* Ny (evdOptions::Ny)       */
    int half_window_x;       /* Nx (evdOptions::Nx)       */
    int method;              /* enum fpl_method           */
    int semantics;           /* enum fpl_semantics        */
    int mini_stack_count;    /* >= 1; reference date = mini_stack_count-1 */
    int band_width;          /* STBAS bandwidth           */
    int min_neighbors;       /* phase_link semantics only */
    int precision;           /* enum fpl_precision        */
    int memory;              /* enum fpl_memory           */
    int row_begin, row_end;
    const void *stack;       /* complex64 [nbands][rows][cols] */
    const uint32_t *nmap;    /* [rows][cols][nulong]           */
    void *phase;             /* complex64 [nbands][rows][cols] */
    float *tcorr;            /* [rows][cols]                   */
    void *comp;              /* complex64 [rows][cols]         */
    int32_t *status;         /* optional [rows][cols]          */
} fpl_job;

/* statistics of the last fpl_run on a context */
typedef struct {
    long long pixels;            /* pixels in the row range          */
    long long fp64_pixels;       /* pixels settled by the FP64 path  */
    long long mixed_fp64_inverse;/* MLE pixels whose |G| inverse ran in FP64 */
    long long slow_path_pixels;  /* pixels that left the fast eigen path (second shift or Householder) */
    float kernel_ms;             /* device time of the compute kernels */
    float total_ms;              /* wall time of the call             */
} fpl_stats;

/* Creates a context on CUDA device `device` (owns a stream and scratch).
 * Replaces the per-run set-up of evd_process (src/evd/evd.cpp:370-393). */
int fpl_ctx_create(int device, fpl_ctx **out);
int fpl_ctx_destroy(fpl_ctx *ctx);

/* Synchronous in-memory run; host or device buffers per job->memory.
 * Replaces the OpenMP pixel loop of evd_process
 * (src/evd/evd.cpp:512-788; src/phase_link/phase_link.cpp:479-666). */
int fpl_run(fpl_ctx *ctx, const fpl_job *job);

/* Asynchronous run on `stream` (a cudaStream_t used as given: NULL is the
 * legacy default stream); device buffers only.  Runs sharing one context
 * share its scratch: each run waits on the GPU for the context's previous
 * run, on whatever stream that was enqueued (inside a stream capture the
 * caller's graph orders them instead).  Same replacement as fpl_run. */
int fpl_run_async(fpl_ctx *ctx, const fpl_job *job, void *stream);

int fpl_last_stats(const fpl_ctx *ctx, fpl_stats *out);

/* ---- batches of jobs ------------------------------------------------------
 * Many device-memory jobs -- scenes or ministacks of different size, stack
 * depth, window and method -- run as one persistent launch per padded depth
 * (16 / 32 / 64 dates), with warps taking pixels dynamically across jobs,
 * followed by one FP64 settle launch.  Replaces running the evd module once
 * per ministack (src/sequential/sequential.py:193-254 calls evd_process in a
 * loop).  FPL_BATCH_GRAPH captures the launch sequence into a CUDA graph at
 * creation; fpl_batch_run replays it (buffers are fixed, their contents may
 * change between runs).  FPL_BATCH_AUTOTUNE times candidate CTA shapes on
 * the batch at creation and caches the fastest per (form, depth, window,
 * mean SHP count) in the context.  Jobs with precision FPL_PREC_MIXED run
 * the mixed form: cut into row pieces, packed into waves of <= 2^20 pixels,
 * one tensor-core Gamma launch over the tiles and one solve launch over the
 * pixels of each wave. */
#define FPL_BATCH_GRAPH 1
#define FPL_BATCH_AUTOTUNE 2
typedef struct fpl_batch fpl_batch;
int fpl_batch_create(fpl_ctx *ctx, const fpl_job *jobs, int njobs, int flags, fpl_batch **out);
int fpl_batch_run(fpl_batch *batch, void *stream);
/* waits for the device; fp64_pixels / slow_path_pixels summed over the jobs */
int fpl_batch_stats(const fpl_batch *batch, fpl_stats *out);
int fpl_batch_destroy(fpl_batch *batch);

/* ---- serving loop -----------------------------------------------------------
 * A request loop for phase-linking jobs (no counterpart in the reference,
 * which runs one module invocation per process).  fpl_server_submit queues a
 * job whose buffers are host memory (valid, and preferably page-locked, until
 * the job is done); a scheduler thread admits jobs in arrival order while
 * their device footprint fits memory_budget, stages them on a copy stream,
 * and runs waves of at most wave_pixels pixels in which every resident job
 * gets a slice of rows -- jobs arriving during a wave join the next one
 * (continuous batching).  Results are copied back as each job finishes.  A
 * job's result does not depend on the other jobs in flight. */
typedef struct fpl_server fpl_server;
typedef struct {
    size_t memory_budget;      /* device bytes for resident jobs (default 80 GB) */
    long long wave_pixels;     /* pixels per wave (default 1048576)             */
    int device;
} fpl_server_config;
typedef struct {
    double queue_ms;           /* submit -> admitted      */
    double run_ms;             /* admitted -> results back */
    double total_ms;           /* submit -> results back   */
    int rc;
} fpl_ticket_info;
void fpl_server_config_default(fpl_server_config *cfg);
int fpl_server_create(const fpl_server_config *cfg, fpl_server **out);
int fpl_server_submit(fpl_server *srv, const fpl_job *job, unsigned long long *ticket);
/* waits up to timeout_s for the job; 0 when its outputs are in place */
int fpl_server_wait(fpl_server *srv, unsigned long long ticket, double timeout_s, fpl_ticket_info *info);
int fpl_server_destroy(fpl_server *srv);

/* ---- run without device allocation (no counterpart in the reference) -----
 * For callers that cannot call cudaMalloc -- an application whose device
 * memory belongs to another allocator, or a service that must not allocate
 * after start-up.  Same job and results as fpl_run_async on device buffers
 * in the plain FP32 form (a job asking for the mixed form runs the FP32 form
 * here: the mixed form's coherence records need gigabytes of scratch), on
 * the current CUDA device, but no context is needed and nothing is
 * allocated: the kernels' scratch is a fixed array inside the library, held
 * by every GPU that loads it until the process exits.  Every call looks up
 * that array's device address in the current CUDA context; the first call
 * in a context (on a device, after a cudaDeviceReset, or in a driver context
 * of the caller's) also loads the library's module there, so make that
 * first call before any stream capture.  A call covers at most
 * FPL_NOALLOC_MAX_PIXELS pixels ((row_end - row_begin) * cols); larger jobs
 * return FPL_ERR_NOALLOC_LIMIT and can be split into row ranges, which give
 * the same results bit for bit.  All calls share the array, so calls whose
 * work overlaps on the GPU race; serialise them on one stream.  A call
 * reports no statistics and no device error flags (the kernels' one flag,
 * FP64 work list full, cannot be raised: the list has an entry for every
 * pixel a call may cover). */
#define FPL_NOALLOC_MAX_PIXELS 524288
int fpl_run_noalloc(const fpl_job *job, void *stream);

/* ---- diagnostics (no counterpart in the reference) ------------------------ */
/* Text of the last CUDA / device error seen by the context. */
const char *fpl_ctx_last_error(const fpl_ctx *ctx);
/* Tuning hooks: width of the FP32 rounding band (in units of n*eps*|A|_F,
 * < 0 keeps the current value) and FP64 for every pixel (test use). */
int fpl_ctx_set_tuning(fpl_ctx *ctx, float amb_scale, int force_fp64);
/* Shifts of the FP32 MLE inverse iteration, as fractions of min(1, rho) (rho
 * the Rayleigh quotient of the start vector): the first attempt and the
 * second one made when M - sigma I is not positive definite (defaults 0.999,
 * 0.97).  A shift above 1 makes that attempt fail, which is how tests reach
 * the second attempt and the Householder path.  Runs and batches on this
 * context use them (servers and fpl_run_noalloc keep the defaults). */
int fpl_ctx_set_shift(fpl_ctx *ctx, float shift, float backoff);
/* Per-kernel device timing of subsequent runs (CUDA events on the run's
 * stream); fpl_ctx_profile waits for them, returns the summed FP32 and FP64
 * kernel milliseconds and the run count, and resets the record. */
int fpl_ctx_set_profiling(fpl_ctx *ctx, int on);
int fpl_ctx_profile(fpl_ctx *ctx, double *fp32_ms, double *fp64_ms, int *runs);
/* Per-kernel split of the runs read by the last fpl_ctx_profile call:
 * ms[tag] for tag < FPL_KTAG_COUNT (the FP32 figure of fpl_ctx_profile is
 * FPL_KTAG_FP32 + FPL_KTAG_GRAM + FPL_KTAG_SOLVE, the FP64 one FPL_KTAG_FP64). */
enum fpl_kernel_tag {
    FPL_KTAG_FP32 = 0,       /* plain FP32 pixel kernel (gather + Gamma + solve) */
    FPL_KTAG_GRAM = 1,       /* mixed form: tensor-core Gamma records            */
    FPL_KTAG_SOLVE = 2,      /* mixed form: eigen-solves from the records        */
    FPL_KTAG_FP64 = 3,       /* FP64 settle pass                                 */
    FPL_KTAG_COUNT = 4
};
int fpl_ctx_profile_kernels(const fpl_ctx *ctx, double *ms, int count);

/* ---- SHP neighbourhood map (the nmap module) --------------------------------
 * The producer of the nmap input: for every pixel, the two-sample
 * Kolmogorov-Smirnov (method FPL_NMAP_KS2) or Anderson-Darling
 * (FPL_NMAP_AD2) test of its N amplitudes against those of each pixel of
 * its (2Ny+1) x (2Nx+1) window; the neighbour's bit is set (Ulongmask layout)
 * when the test's probability is >= prob, and the centre bit of every valid
 * pixel.  Each pair is tested with the reference's argument order (the pixel
 * whose half-window loop reaches the other is the first sample), which
 * matters for AD2 when the samples share values.  A pixel is valid when the optional mask is nonzero and all its
 * amplitudes |x_b| / alpha_b are nonzero and not NaN, alpha_b being the
 * band's "amplitudeConstant" normalised to the first band (<= 0 or absent:
 * 1).  Replaces the in-memory core of nmap_process (src/nmap/nmap.cpp:
 * 345-473; nmapOptions::method "KS2" / "AD2", src/nmap/nmap.cpp:27-40,
 * src/nmap/KS2sample.hpp:96-144, src/nmap/AD2unique.hpp:270-347).  Returns
 * FPL_ERR_OPTIONS when prob lies within rounding of one of the KS test's
 * discrete probability values for this stack depth, or of the AD test's
 * p-value at its decision boundary (move it by 1e-12). */
#define FPL_NMAP_KS2 0
#define FPL_NMAP_AD2 1
typedef struct {
    int rows, cols, nbands;
    int half_window_y, half_window_x;    /* nmapOptions::Ny, Nx (default 5, 5) */
    double prob;                         /* nmapOptions::prob (default 0.05) */
    int memory;                          /* enum fpl_memory */
    const void *stack;                   /* complex64 [nbands][rows][cols]        */
    const uint8_t *mask;                 /* optional [rows][cols], 0 = excluded   */
    const double *amp_const;             /* optional [nbands], host memory        */
    uint32_t *nmap;                      /* out [rows][cols][nulong]              */
    int32_t *count;                      /* optional out [rows][cols]: bits set   */
    int method;                          /* FPL_NMAP_KS2 (default 0) or FPL_NMAP_AD2 */
} fpl_nmap_job;

int fpl_nmap(fpl_ctx *ctx, const fpl_nmap_job *job);

/* ---- file-level module call ------------------------------------------------
 * Mirrors evdOptions (src/evd/evd.hpp:19-54; src/phase_link/phase_link.hpp:20-57)
 * and evd_process(evdOptions*) (src/evd/evd.cpp:16-888;
 * src/phase_link/phase_link.cpp:17-755): reads a VRT / ENVI stack whose bands
 * carry a "Date" item in metadata domain "slc", an ENVI nmap with
 * HALFWINDOWX / HALFWINDOWY, and writes <date>.slc, tcorr.bin and the
 * compressed SLC as ENVI BIP files.                                          */
typedef struct {
    const char *inputDS;                 /* stack VRT or ENVI file        */
    const char *wtsDS;                   /* nmap ENVI file                */
    const char *outputFolder;
    const char *outputCompressedSlcFolder;   /* NULL: outputFolder   */
    const char *compSlc;                 /* NULL: "compslc.bin"           */
    int blocksize;                       /* default 64                    */
    int memsize;                         /* MB, default 2048              */
    int Nx, Ny;                          /* default 5, 5                  */
    int minNeighbors;                    /* default 2                     */
    int miniStackCount;                  /* default 1                     */
    const char *method;                  /* "MLE" / "EVD" / "STBAS"       */
    int bandWidth;                       /* default -1                    */
    int semantics;                       /* enum fpl_semantics            */
    int precision;                       /* enum fpl_precision            */
    int device;                          /* CUDA device                   */
    int verbose;                         /* print like the reference      */
} fpl_options;

/* Fills the defaults of evdOptions::evdOptions (src/evd/evd.hpp:58-68). */
void fpl_options_default(fpl_options *opts);

/* File-level run; returns 0 or the reference's module codes. */
int fpl_process(const fpl_options *opts);

/* Wrapped-phase datum adjustment of the sequential estimator: for the
 * ndates dates of one ministack, out[d][p] = phase[d][p] * datum[p]
 * (complex64, product in double).  Replaces the derived VRT band with pixel
 * function "mul" that python/adjustMiniStacks.py:174-197 writes per date
 * (called from adjust_wrapped, :203-223).  Device pointers; enqueued on
 * `stream` (NULL = the legacy default stream); out may alias phase. */
int fpl_adjust_wrapped(fpl_ctx *ctx, const void *phase, const void *datum, void *out,
                       int ndates, long long npix, void *stream);

/* PS/DS merge of python/integratePS.py (integratePS2DS :94-126,
 * get_fullres_ifgram :66-75, getCoherence :129-152) over the single-master
 * network of python/Network.py:95-104.  For every band j != master, in band
 * order (output slot q = j - (j > master)):
 *   ifg[q][p] = ds[j][p] * conj(ds[master][p])                      (DS pixel)
 *             = exp(1j * angle(slc[j][p] * conj(slc[master][p])))  (ps[p] == 1)
 * and tcorr_out[p] = 0.95 at PS pixels, tcorr[p] elsewhere.  Device
 * pointers; enqueued on `stream` (NULL = the legacy default stream).
 * tcorr_out may alias tcorr; ifg must not overlap the inputs.  An empty
 * scene (rows or cols 0) returns FPL_OK without reading any pointer. */
typedef struct fpl_ps_job {
    int rows, cols, nbands;
    int master;                  /* band of the reference date (the first date: 0) */
    const void *ds;              /* complex64 [nbands][rows][cols], phase-linked stack */
    const void *slc;             /* complex64 [nbands][rows][cols], SLC stack          */
    const float *tcorr;          /* [rows][cols] temporal coherence                   */
    const uint8_t *ps;           /* [rows][cols] PS map, 1 = PS pixel                 */
    void *ifg;                   /* complex64 [nbands-1][rows][cols]                  */
    float *tcorr_out;            /* [rows][cols]                                      */
} fpl_ps_job;
int fpl_integrate_ps(fpl_ctx *ctx, const fpl_ps_job *job, void *stream);

/* Human-readable text for a return code. */
const char *fpl_error_string(int code);

/* Library version string. */
const char *fpl_version(void);

#ifdef __cplusplus
}
#endif
#endif
