// kernels.h -- host-side declarations of the kernel launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fpl {

struct KParams;
struct BoxSeg;
struct BatchEntry;

// padded order used for a stack depth (16, 32, 64; 0 = unsupported)
int pick_np(int nb);

// plain FP32 form over P.npix pixels starting at P.pix_begin
cudaError_t launch_fp32(const KParams &P, int num_sms, cudaStream_t st);

// FP64 form over the work list in P (or over every pixel if P.fb_list is null)
cudaError_t launch_fp64(const KParams &P, int num_sms, cudaStream_t st);

// mixed form: is the tensor-core Gamma kernel available for this stack
// depth and window (nbands <= 64, window width <= 63, window union of an
// 8 x 16 pixel tile <= 2048 samples)
bool gram_box_supported(int nb, int ny, int nx);

// floats per Gamma record written by launch_gram_box
int gram_box_record(int nb);

// mixed form: tensor-core Gamma records for the whole rows
// [P.pix_begin, P.pix_begin + P.npix) into P.cbuf / P.cinfo
cudaError_t launch_gram_box(const KParams &P, int num_sms, cudaStream_t st);

// mixed form: eigen-solves and outputs from P.cbuf / P.cinfo
cudaError_t launch_solve(const KParams &P, int num_sms, cudaStream_t st);

// batched mixed form: a launch of the Gamma kernel covers gram_box_tiles(P)
// tiles and needs gram_box_smem bytes of shared memory.
long long gram_box_tiles(const KParams &P);
size_t gram_box_smem(int nb, int ny, int nx);
// tiles of every segment in one persistent launch (smem: the largest
// gram_box_smem of the segments)
cudaError_t launch_gram_batch(const BoxSeg *segs, int nseg, long long total, size_t smem,
                              int num_sms, cudaStream_t st);
// kernel attributes of the batched mixed form for padded depth np (call
// before capturing a launch sequence)
cudaError_t prepare_mixed_batch(int np);
cudaError_t prepare_gram_batch();
// eigen-solves of every entry (one padded depth np) in one persistent launch;
// warps: warps per CTA (0 = the most that fit; see solve_max_warps)
cudaError_t launch_solve_batch(int np, const BatchEntry *ents, int nent, long long total, int num_sms,
                               cudaStream_t st, int warps = 0);
int solve_max_warps(int np);

}  // namespace fpl
