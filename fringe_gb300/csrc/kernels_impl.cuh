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

// mixed form, second half: eigen-solves from the tensor-core Gamma records.
// TM: each warp keeps its pixel's coherence rows in tensor memory (2*NP
// columns of its 32-lane quadrant) instead of shared memory, so a CTA holds
// about twice as many warps; the kernel issues no MMA.
__device__ __forceinline__ int tmem_cols_for(int warps, int np)
{
    int need = ((warps + 3) / 4) * 2 * np, cols = 32;
    while (cols < need) cols <<= 1;
    return cols;
}

template <int NP, bool TM>
__global__ void __launch_bounds__(TM ? 640 : 512, 1) k_solve(KParams P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr size_t per_warp = TM ? Lay<float, NP>::bytes_noc : Lay<float, NP>::bytes;
    unsigned char *sm = smem + (size_t)warp * per_warp;
    const long long gw = (long long)blockIdx.x * warps + warp;
    const long long nw = (long long)gridDim.x * warps;
    if constexpr (TM) {
        __shared__ uint32_t tslot;
        const int tcols = tmem_cols_for(warps, NP);
        if (warp == 0) {
            asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                         :: "r"((uint32_t)__cvta_generic_to_shared(&tslot)), "r"(tcols) : "memory");
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t tbase = tslot;
        const CRowsTmem<NP> cp{tbase + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)((warp >> 2) * 2 * NP)};
        C2<float> *A = reinterpret_cast<C2<float> *>(sm + Lay<float, NP>::wm);
        for (long long q = gw; q < P.npix; q += nw) {
            const long long pp = P.pix_begin + q;
            const int npix = pixel_load_gamma<NP, false>(P, pp, sm, lane, A);
            if (npix >= 0 && rows_coherence<NP>(P, pp, A, sm, cp, lane))
                pixel_solve<float, NP>(P, pp, sm, lane, npix, cp);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (warp == 0) {
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(tcols) : "memory");
        }
    } else {
        C2<float> *Cm = reinterpret_cast<C2<float> *>(sm + Lay<float, NP>::cm);
        const CRowsSmem<float, NP> cp{Cm, lane};
        for (long long q = gw; q < P.npix; q += nw) {
            const long long pp = P.pix_begin + q;
            const int npix = pixel_load_gamma<NP>(P, pp, sm, lane, Cm);
            if (npix >= 0) pixel_solve<float, NP>(P, pp, sm, lane, npix, cp);
        }
    }
}

template <int NP, bool TM>
static cudaError_t launch_solve_t(const KParams &P, int num_sms, cudaStream_t st)
{
    static bool configured[64] = {false};
    const size_t per_warp = TM ? Lay<float, NP>::bytes_noc : Lay<float, NP>::bytes;
    const size_t budget = 224 * 1024;
    const int cap = TM ? 32 : 16;
    int warps = int(budget / per_warp);
    if (warps > cap) warps = cap;
    if (warps < 1) warps = 1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !configured[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_solve<NP, TM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)budget);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(k_solve<NP, TM>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        if (e != cudaSuccess) return e;
        configured[dev] = true;
    }
    // registers can bound the warps of a CTA below the shared-memory figure
    int per_sm = 0;
    size_t smem = per_warp * warps;
    for (;;) {
        smem = per_warp * warps;
        // one CTA per SM in the tensor-memory form: at least half the shared
        // memory, so a second CTA never waits on a tensor-memory allocation
        if (TM && smem < budget / 2 + 1024) smem = budget / 2 + 1024;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_solve<NP, TM>, warps * 32, smem);
        if (e != cudaSuccess) return e;
        if (per_sm >= 1 || warps == 1) break;
        --warps;
    }
    if (per_sm < 1) per_sm = 1;
    if (TM) per_sm = 1;
    long long blocks = (long long)num_sms * per_sm;
    long long need = (P.npix + warps - 1) / warps;
    if (need < blocks) blocks = need > 0 ? need : 1;
    k_solve<NP, TM><<<(unsigned)blocks, warps * 32, smem, st>>>(P);
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
