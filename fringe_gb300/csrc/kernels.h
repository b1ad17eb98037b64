// kernels.h -- host-side declarations of the kernel launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fpl {

struct KParams;

// padded order used for a stack depth (16, 32, 64; 0 = unsupported)
int pick_np(int nb);

// plain FP32 form over P.npix pixels starting at P.pix_begin
cudaError_t launch_fp32(const KParams &P, int num_sms, cudaStream_t st);

// FP64 form over the work list in P (or over every pixel if P.fb_list is null)
cudaError_t launch_fp64(const KParams &P, int num_sms, cudaStream_t st);

// mixed form: tensor-core coherence matrices for P.npix pixels from
// P.pix_begin into P.cbuf / P.cinfo (nbands <= 32)
cudaError_t launch_gram_tc(const KParams &P, int num_sms, cudaStream_t st);

// mixed form: eigen-solves and outputs from P.cbuf / P.cinfo
cudaError_t launch_solve(const KParams &P, int num_sms, cudaStream_t st);

}  // namespace fpl
