// integrate.cu -- the PS/DS merge of python/integratePS.py on the GPU.
//
// For the single-master network (python/Network.py:95-104) the reference
// writes, per pair (master, j), the interferogram of the phase-linked stack
// ds_j * conj(ds_master) (integratePS2DS, python/integratePS.py:94-126),
// replaced at PS pixels (map value 1) by exp(1j * angle(slc_j *
// conj(slc_master))) of the original SLCs (get_fullres_ifgram, :66-75), and
// the temporal coherence with PS pixels set to 0.95 (getCoherence,
// :129-152).  Every value is per pixel, so the reference's blocks of lines
// need no counterpart: one thread per pixel walks the dates, reading the one
// stack the pixel uses.  HBM-bound: per pixel 8 bytes per date in and out.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "fringe_gb300.h"
#include "guard.h"
#include "ctx.h"

namespace {

// x * conj(m) with the fused multiply-adds of NumPy's vectorised complex64
// loop: re = fma(x.re, m.re, x.im * m.im), im = fma(x.im, m.re, -(x.re * m.im))
__device__ __forceinline__ float2 mul_conj(float2 x, float2 m)
{
    return make_float2(__fmaf_rn(x.x, m.x, __fmul_rn(x.y, m.y)), __fmaf_rn(x.y, m.x, -__fmul_rn(x.x, m.y)));
}

// exp(1j * angle(o)): o / |o| for a normal, finite |o|^2 (within a few ulp
// of cos / sin of the angle); zero, tiny, huge or non-finite products take
// atan2 + sincos, which keep angle's conventions (angle(+-0 + -0j) = +-pi,
// angle(0) = 0)
__device__ __forceinline__ float2 unit_phasor(float2 o)
{
    const float r2 = fmaf(o.x, o.x, o.y * o.y);
    if (r2 >= 1.17549435e-38f && r2 <= 3.40282347e38f) {
        const float r = rsqrtf(r2);
        return make_float2(o.x * r, o.y * r);
    }
    float sn, cs;
    sincosf(atan2f(o.y, o.x), &sn, &cs);
    return make_float2(cs, sn);
}

__global__ void k_integrate_ps(const float2 *__restrict__ ds, const float2 *__restrict__ slc,
                               const float *tcorr, const uint8_t *__restrict__ ps, float2 *__restrict__ ifg,
                               float *tc_out, int nb, int master, long long npix)
{
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix;
         p += (long long)gridDim.x * blockDim.x) {
        const bool is_ps = ps[p] == 1;
        const float t = tcorr[p];
        tc_out[p] = is_ps ? 0.95f : t;
        const float2 *src = is_ps ? slc : ds;
        const float2 m = src[(long long)master * npix + p];
        // four dates' samples in flight before their results are stored
        for (int j0 = 0; j0 < nb; j0 += 4) {
            float2 x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                x[u] = (j0 + u < nb) ? src[(long long)(j0 + u) * npix + p] : make_float2(0.f, 0.f);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int j = j0 + u;
                if (j >= nb || j == master) continue;
                float2 o = mul_conj(x[u], m);
                if (is_ps) o = unit_phasor(o);
                ifg[(long long)(j - (j > master)) * npix + p] = o;
            }
        }
    }
}

}  // namespace

extern "C" int fpl_integrate_ps(fpl_ctx *ctx, const fpl_ps_job *job, void *stream)
{
    return fpl_guard([&]() -> int {
        if (!ctx || !job) return FPL_ERR_NULL;
        if (job->rows < 0 || job->cols < 0 || job->nbands < 1 || job->master < 0 || job->master >= job->nbands)
            return FPL_ERR_OPTIONS;
        const long long npix = (long long)job->rows * job->cols;
        if (npix == 0) return FPL_OK;             // empty scene: no buffer is touched
        if (!job->ds || !job->slc || !job->tcorr || !job->ps || !job->tcorr_out || (job->nbands > 1 && !job->ifg))
            return FPL_ERR_NULL;
        cudaError_t e = cudaSetDevice(ctx->device);
        if (e == cudaSuccess) {
            const long long blocks = std::min<long long>((npix + 255) / 256, (long long)ctx->num_sms * 8);
            k_integrate_ps<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
                static_cast<const float2 *>(job->ds), static_cast<const float2 *>(job->slc), job->tcorr, job->ps,
                static_cast<float2 *>(job->ifg), job->tcorr_out, job->nbands, job->master, npix);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) {
            ctx->last_error = std::string("fpl_integrate_ps: ") + cudaGetErrorString(e);
            return FPL_ERR_CUDA;
        }
        return FPL_OK;
    });
}
