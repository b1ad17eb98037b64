// kernels_impl.cuh -- pixel kernels and their launchers (included by
// kernels_f32.cu and kernels_f64.cu so the two precisions compile in parallel).
//
// k_pixels<float, NP>  : plain FP32 form over a contiguous pixel range.
// k_pixels<double, NP> : FP64 form over the work list written by the FP32
//                        pass (pixels whose discrete decisions fall inside the
//                        FP32 rounding band), or over every pixel when no list
//                        is given (used to check the FP64 form itself).
// Both are persistent: the grid is sized to the resident capacity of the
// GPU and warps stride over their pixels.
#pragma once
#include "kernels.h"
#include "pixel.cuh"

namespace fpl {

template <typename T, int NP>
__global__ void k_pixels(KParams P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *sm = smem + (size_t)warp * Lay<T, NP>::bytes;
    const long long gw = (long long)blockIdx.x * warps + warp;
    const long long nw = (long long)gridDim.x * warps;
    if (sizeof(T) == 4 || P.fb_list == nullptr) {
        for (long long q = gw; q < P.npix; q += nw) process_pixel<T, NP>(P, P.pix_begin + q, sm, lane);
    } else {
        int cnt = *((volatile int *)P.fb_count);
        cnt = cnt < P.fb_cap ? cnt : P.fb_cap;
        for (long long q = gw; q < cnt; q += nw) process_pixel<T, NP>(P, P.fb_list[q], sm, lane);
    }
}

// mixed form, second half: eigen-solves from the tensor-core Gamma records
template <int NP>
__global__ void k_solve(KParams P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *sm = smem + (size_t)warp * Lay<float, NP>::bytes;
    const long long gw = (long long)blockIdx.x * warps + warp;
    const long long nw = (long long)gridDim.x * warps;
    for (long long q = gw; q < P.npix; q += nw) {
        const long long pp = P.pix_begin + q;
        const int npix = pixel_load_gamma<NP>(P, pp, sm, lane);
        if (npix >= 0) pixel_solve<float, NP>(P, pp, sm, lane, npix);
    }
}

template <int NP>
static cudaError_t launch_solve_t(const KParams &P, int num_sms, cudaStream_t st)
{
    static bool configured[64] = {false};
    const size_t per_warp = Lay<float, NP>::bytes;
    const size_t budget = 224 * 1024;
    int warps = int(budget / per_warp);
    if (warps > 16) warps = 16;
    if (warps < 1) warps = 1;
    const size_t smem = per_warp * warps;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !configured[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_solve<NP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(k_solve<NP>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        if (e != cudaSuccess) return e;
        configured[dev] = true;
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve<NP>, warps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    long long blocks = (long long)num_sms * per_sm;
    long long need = (P.npix + warps - 1) / warps;
    if (need < blocks) blocks = need > 0 ? need : 1;
    k_solve<NP><<<(unsigned)blocks, warps * 32, smem, st>>>(P);
    return cudaGetLastError();
}

template <typename T, int NP>
static cudaError_t launch_t(const KParams &P, int num_sms, cudaStream_t st)
{
    static bool configured[64] = {false};
    const size_t per_warp = Lay<T, NP>::bytes;
    const size_t budget = 224 * 1024;   // of the 227 KB a block may opt into
    int warps = int(budget / per_warp);
    if (warps > 16) warps = 16;
    if (warps < 1) warps = 1;
    const size_t smem = per_warp * warps;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !configured[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_pixels<T, NP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(k_pixels<T, NP>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        if (e != cudaSuccess) return e;
        configured[dev] = true;
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pixels<T, NP>, warps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    long long work = P.npix;
    long long blocks = (long long)num_sms * per_sm;
    long long need = (work + warps - 1) / warps;
    if (sizeof(T) == 4 && need < blocks) blocks = need > 0 ? need : 1;
    k_pixels<T, NP><<<(unsigned)blocks, warps * 32, smem, st>>>(P);
    return cudaGetLastError();
}

}  // namespace fpl
