// batch.h -- shared pieces of the batch launch (batch.cu) used by the
// serving loop (serve.cu).
#pragma once

#include <cuda_runtime.h>

#include "fringe_gb300.h"
#include "pixel.cuh"

namespace fpl {

// warps per CTA that fit the shared-memory budget for a padded depth
int max_warps(int np, bool fp64);
// function attributes (dynamic shared memory, carveout) of the batch kernels
cudaError_t configure_np(int np);
// persistent FP32 launch over `total` pixels of `njobs` entries of one depth class
cudaError_t launch_batch(int np, const BatchEntry *jobs, int njobs, long long total,
                         unsigned long long *counter, int warps, int num_sms, cudaStream_t st);
// persistent FP64 settle launch over the work lists of `njobs` entries
cudaError_t launch_batch64(int np, const BatchEntry *jobs, int njobs, int num_sms, cudaStream_t st);
// KParams of job rows [r0, r1) (counters and work list left unset)
void fill_params(KParams &P, const fpl_job &jb, int r0, int r1, float amb, float cond_max);

}  // namespace fpl
