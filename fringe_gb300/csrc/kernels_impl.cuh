// kernels_impl.cuh -- pixel kernels and their launchers (included by
// kernels_f32.cu and kernels_f64.cu so the two precisions compile in parallel).
//
// k_pixels<float, NP>  : plain FP32 form over a contiguous pixel range.
// k_pixels<double, NP> : FP64 form over the work list written by the FP32
//                        pass (pixels whose discrete decisions fall inside the
//                        FP32 rounding band), or over every pixel when no list
//                        is given (used to check the FP64 form itself).
// Both are persistent: the grid is sized to the resident capacity of the
// GPU; warps stride over a pixel range, or draw work-list entries from a
// cursor.
#pragma once
#include <type_traits>
#include "kernels.h"
#include "pixel.cuh"
#include "solve_pair.cuh"

namespace fpl {

template <typename T, int NP>
__global__ void k_pixels(KParams P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *sm = smem + (size_t)warp * KPixWarp<T, NP>::bytes;
    const long long gw = (long long)blockIdx.x * warps + warp;
    const long long nw = (long long)gridDim.x * warps;
    // C in tensor memory: FP64 at 64 dates (one lane quadrant per warp) and
    // FP32 at <= 32 dates (2*NP columns of the warp's quadrant per warp)
    __shared__ uint32_t tslot;
    uint32_t tbase = 0, taddr = 0;
    int tcols = 0;
    if constexpr (CInTmem<T, NP>::value) {
        tcols = 512;
        tbase = tmem_alloc_cta(&tslot, warp, tcols);
        taddr = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
    } else if constexpr (CRowsTmemF<T, NP>::value) {
        tcols = tmem_cols_for(warps, NP);
        tbase = tmem_alloc_cta(&tslot, warp, (uint32_t)tcols);
        taddr = tbase + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(warp >> 2) * CRowsTmem<NP>::kColsPerWarp;
    }
    if (sizeof(T) == 4 || P.fb_list == nullptr) {
        for (long long q = gw; q < P.npix; q += nw) process_pixel<T, NP>(P, P.pix_begin + q, sm, lane, taddr);
    } else {
        int cnt = *((volatile int *)P.fb_count);
        cnt = cnt < P.fb_cap ? cnt : P.fb_cap;
        for (long long q = fb_next(P, lane); q < cnt; q = fb_next(P, lane))
            process_pixel<T, NP>(P, P.fb_list[q], sm, lane, taddr);
    }
    if constexpr (CInTmem<T, NP>::value || CRowsTmemF<T, NP>::value) tmem_free_cta(tbase, warp, (uint32_t)tcols);
}

// mixed form, second half: eigen-solves from the tensor-core Gamma records.
// TM: each warp keeps its pixel's coherence rows in tensor memory (2*NP
// columns of its 32-lane quadrant) instead of shared memory, so a CTA holds
// about twice as many warps; the kernel issues no MMA.  At padded order 16 a
// warp solves two pixels, one per 16-lane half (solve_pair.cuh): two slabs
// per warp, the rows of both in the warp's 2*NP columns.
template <int NP, bool TM> struct PairSolve {
    static constexpr bool value = TM && NP == 16;
};
template <int NP, bool TM> struct SolveWarp {
    static constexpr bool pair = PairSolve<NP, TM>::value;
    static constexpr size_t bytes =
        pair ? 2 * Lay<float, NP>::bytes_noc : (TM ? Lay<float, NP>::bytes_noc : Lay<float, NP>::bytes);
    // warp work items: pixel pairs or pixels
    static __host__ __device__ long long items(long long px) { return pair ? (px + 1) / 2 : px; }
};

// pixel pp of the launch P: record -> coherence rows -> solve and outputs
template <int NP, typename CP>
__device__ __forceinline__ void solve_pixel(const KParams &P, long long pp, unsigned char *sm, int lane, const CP &cp,
                                            C2<float> *A)
{
    if constexpr (NP <= 32) {
        const int npix = pixel_load_gamma<NP, false>(P, pp, sm, lane, A);
        float cfro = -1.f;
        if (npix >= 0 && rows_coherence<NP>(P, pp, A, sm, cp, lane, &cfro))
            pixel_solve<float, NP>(P, pp, sm, lane, npix, cp, cfro);
    } else if constexpr (std::is_same<CP, CRowsTmem<NP>>::value) {
        // two rows per lane: normalise in the slab, then copy the rows over
        const int npix = pixel_load_gamma<NP>(P, pp, sm, lane, A);
        if (npix >= 0) {
            rows_from_smem<NP>(cp, A, lane);
            pixel_solve<float, NP>(P, pp, sm, lane, npix, cp);
        }
    } else {
        const int npix = pixel_load_gamma<NP>(P, pp, sm, lane, A);
        if (npix >= 0) pixel_solve<float, NP>(P, pp, sm, lane, npix, cp);
    }
}

// Solve kernel over a pixel source: SRC(q) gives (launch, pixel) of item q
// of [0, total).  TM: each warp keeps its pixel's coherence rows in tensor
// memory (2*NP columns of its 32-lane quadrant) instead of shared memory,
// so a CTA holds about twice as many warps; the kernel issues no MMA.
template <int NP, bool TM, typename SRC>
__device__ __forceinline__ void solve_loop(long long total, const SRC &src)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr size_t per_warp = SolveWarp<NP, TM>::bytes;
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
        const CRowsTmem<NP> cp{tbase + ((uint32_t)(32 * (warp & 3)) << 16) +
                               (uint32_t)(warp >> 2) * CRowsTmem<NP>::kColsPerWarp};
        C2<float> *A = reinterpret_cast<C2<float> *>(sm + Lay<float, NP>::wm);
        if constexpr (PairSolve<NP, TM>::value) {
            // pixels 2k and 2k+1 on halves 0 and 1; MLE pixels with evd
            // semantics are solved by the halves together, any other pixel by
            // the whole warp on its half's slab
            const int h = lane >> 4;
            const PairHalf H{lane & 15, h, h ? 0xffff0000u : 0x0000ffffu};
            const long long npair = (total + 1) >> 1;
            for (long long k = gw; k < npair; k += nw) {
                const long long q0 = 2 * k;
                const bool valid = q0 + h < total;
                long long pp;
                const KParams &P = src(valid ? q0 + h : q0, pp);
                const bool paired = valid && P.method == M_MLE && P.semantics != SEM_PL;
                if (k + nw < npair && q0 + 2 * nw + h < total) {
                    long long pn;
                    const KParams &Pn = src(q0 + 2 * nw + h, pn);
                    pair_prefetch(Pn, pn, H.hl);
                }
                pair_mle(P, pp, sm, cp, H, paired);
                for (int hh = 0; hh < 2; ++hh) {
                    if (!__shfl_sync(0xffffffffu, (int)(valid && !paired), 16 * hh)) continue;
                    long long ph;
                    const KParams &Ph = src(q0 + hh, ph);
                    unsigned char *smh = sm + hh * Lay<float, NP>::bytes_noc;
                    solve_pixel<NP>(Ph, ph, smh, lane, cp, reinterpret_cast<C2<float> *>(smh + Lay<float, NP>::wm));
                }
            }
        } else {
        for (long long q = gw; q < total; q += nw) {
            long long pp;
            const KParams &P = src(q, pp);
            if (q + nw < total) {
                long long pn;
                const KParams &Pn = src(q + nw, pn);
                prefetch_record(Pn, pn, lane);
            }
            solve_pixel<NP>(P, pp, sm, lane, cp, A);
        }
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
        for (long long q = gw; q < total; q += nw) {
            long long pp;
            const KParams &P = src(q, pp);
            if (q + nw < total) {
                long long pn;
                const KParams &Pn = src(q + nw, pn);
                prefetch_record(Pn, pn, lane);
            }
            solve_pixel<NP>(P, pp, sm, lane, cp, Cm);
        }
    }
}

template <int NP, bool TM>
__global__ void __launch_bounds__((TM && NP <= 32) ? 640 : (TM ? 256 : 512), 1) k_solve(KParams P)
{
    solve_loop<NP, TM>(P.npix, [&](long long q, long long &pp) -> const KParams & {
        pp = P.pix_begin + q;
        return P;
    });
}

// the mixed form over many launches of one padded depth
template <int NP, bool TM>
__global__ void __launch_bounds__((TM && NP <= 32) ? 640 : (TM ? 256 : 512), 1) k_solve_batch(const BatchEntry *__restrict__ ents, int nent,
                                                                  long long total)
{
    solve_loop<NP, TM>(total, [&](long long q, long long &pp) -> const KParams & {
        int lo = 0, hi = nent - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (ents[mid].px_offset <= q) lo = mid; else hi = mid - 1;
        }
        pp = ents[lo].P.pix_begin + (q - ents[lo].px_offset);
        return ents[lo].P;
    });
}

// CTA shape of the solve kernels: warps per CTA by shared memory (and
// registers), one CTA per SM in the tensor-memory form
template <int NP, bool TM, typename K>
static cudaError_t solve_shape(K kern, int *warps_out, int *per_sm_out, size_t *smem_out, int warps_req = 0)
{
    const size_t per_warp = SolveWarp<NP, TM>::bytes;
    const size_t budget = 224 * 1024;
    // tensor memory: 512 columns per lane quadrant, CRowsTmem<NP>::kColsPerWarp per warp
    const int cap = TM ? int(4 * (512 / CRowsTmem<NP>::kColsPerWarp)) : 16;
    int warps = int(budget / per_warp);
    if (warps > cap) warps = cap;
    if (warps_req > 0 && warps > warps_req) warps = warps_req;
    if (warps < 1) warps = 1;
    int per_sm = 0;
    size_t smem = per_warp * warps;
    for (;;) {
        smem = per_warp * warps;
        // one CTA per SM in the tensor-memory form: at least half the shared
        // memory, so a second CTA never waits on a tensor-memory allocation
        if (TM && smem < budget / 2 + 1024) smem = budget / 2 + 1024;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem);
        if (e != cudaSuccess) return e;
        if (per_sm >= 1 || warps == 1) break;
        --warps;
    }
    if (per_sm < 1) per_sm = 1;
    if (TM) per_sm = 1;
    *warps_out = warps;
    *per_sm_out = per_sm;
    *smem_out = smem;
    return cudaSuccess;
}

template <typename K>
static cudaError_t solve_configure(K kern, bool *configured)
{
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && configured[dev]) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 224 * 1024);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    if (dev < 64) configured[dev] = true;
    return cudaSuccess;
}

template <int NP, bool TM>
static cudaError_t launch_solve_t(const KParams &P, int num_sms, cudaStream_t st)
{
    static bool configured[64] = {false};
    cudaError_t e = solve_configure(k_solve<NP, TM>, configured);
    if (e != cudaSuccess) return e;
    int warps = 0, per_sm = 0;
    size_t smem = 0;
    if ((e = solve_shape<NP, TM>(k_solve<NP, TM>, &warps, &per_sm, &smem)) != cudaSuccess) return e;
    long long blocks = (long long)num_sms * per_sm;
    long long need = (SolveWarp<NP, TM>::items(P.npix) + warps - 1) / warps;
    if (need < blocks) blocks = need > 0 ? need : 1;
    k_solve<NP, TM><<<(unsigned)blocks, warps * 32, smem, st>>>(P);
    return cudaGetLastError();
}

// attributes of k_solve_batch<NP, TM>, set once per device
template <int NP, bool TM>
static cudaError_t configure_solve_batch()
{
    static bool configured[64] = {false};
    return solve_configure(k_solve_batch<NP, TM>, configured);
}

// warps_req > 0: at most that many warps per CTA (the batch autotuner's
// candidates); 0: as many as shared memory and registers allow
template <int NP, bool TM>
static cudaError_t launch_solve_batch_t(const BatchEntry *ents, int nent, long long total, int num_sms,
                                       cudaStream_t st, int warps_req)
{
    cudaError_t e = configure_solve_batch<NP, TM>();
    if (e != cudaSuccess) return e;
    int warps = 0, per_sm = 0;
    size_t smem = 0;
    if ((e = solve_shape<NP, TM>(k_solve_batch<NP, TM>, &warps, &per_sm, &smem, warps_req)) != cudaSuccess) return e;
    long long blocks = (long long)num_sms * per_sm;
    long long need = (SolveWarp<NP, TM>::items(total) + warps - 1) / warps;
    if (need < blocks) blocks = need > 0 ? need : 1;
    k_solve_batch<NP, TM><<<(unsigned)blocks, warps * 32, smem, st>>>(ents, nent, total);
    return cudaGetLastError();
}

template <typename T, int NP>
static cudaError_t launch_t(const KParams &P, int num_sms, cudaStream_t st)
{
    static bool configured[64] = {false};
    const size_t per_warp = KPixWarp<T, NP>::bytes;
    const size_t budget = 224 * 1024;   // of the 227 KB a block may opt into
    int warps = int(budget / per_warp);
    if (warps > 16) warps = 16;
    if (CInTmem<T, NP>::value && warps > 4) warps = 4;   // one tensor-memory lane quadrant per warp
    // and no more threads than the kernel's registers allow in one CTA
    static int max_threads[64] = {0};
    {
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev < 64 && !max_threads[dev]) {
            cudaFuncAttributes fa;
            cudaError_t e = cudaFuncGetAttributes(&fa, k_pixels<T, NP>);
            if (e != cudaSuccess) return e;
            max_threads[dev] = fa.maxThreadsPerBlock;
        }
        const int lim = (dev < 64 ? max_threads[dev] : 1024) / 32;
        if (warps > lim) warps = lim;
    }
    if (warps < 1) warps = 1;
    size_t smem = per_warp * warps;
    // tensor-memory rows: one CTA per SM (at least half the shared memory),
    // so a second CTA never waits on a tensor-memory allocation
    constexpr bool one_cta = CInTmem<T, NP>::value || CRowsTmemF<T, NP>::value;
    if (one_cta && smem < budget / 2 + 1024) smem = budget / 2 + 1024;
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
    if (per_sm < 1 || one_cta) per_sm = 1;
    long long work = P.npix;
    long long blocks = (long long)num_sms * per_sm;
    long long need = (work + warps - 1) / warps;
    if (sizeof(T) == 4 && need < blocks) blocks = need > 0 ? need : 1;
    k_pixels<T, NP><<<(unsigned)blocks, warps * 32, smem, st>>>(P);
    return cudaGetLastError();
}

}  // namespace fpl
