// kernels_f32.cu -- FP32 instantiations of the pixel kernels.
#include <algorithm>

#include "kernels_impl.cuh"

namespace fpl {

int pick_np(int nb)
{
    if (nb <= 16) return 16;
    if (nb <= 32) return 32;
    if (nb <= 64) return 64;
    return 0;
}

cudaError_t launch_fp32(const KParams &P, int num_sms, cudaStream_t st)
{
    switch (pick_np(P.nb)) {
    case 16: return launch_t<float, 16>(P, num_sms, st);
    case 32: return launch_t<float, 32>(P, num_sms, st);
    case 64: return launch_t<float, 64>(P, num_sms, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_solve(const KParams &P, int num_sms, cudaStream_t st)
{
    switch (pick_np(P.nb)) {
    case 16: return launch_solve_t<16, true>(P, num_sms, st);
    case 32: return launch_solve_t<32, true>(P, num_sms, st);
    case 64: return launch_solve_t<64, true>(P, num_sms, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t prepare_mixed_batch(int np)
{
    cudaError_t e = prepare_gram_batch();
    if (e != cudaSuccess) return e;
    switch (np) {
    case 16: return configure_solve_batch<16, true>();
    case 32: return configure_solve_batch<32, true>();
    case 64: return configure_solve_batch<64, true>();
    }
    return cudaErrorInvalidValue;
}

int solve_max_warps(int np)
{
    switch (np) {
    case 16: return std::min(20, int((224 * 1024) / SolveWarp<16, true>::bytes));
    case 32: return std::min(32, int((224 * 1024) / Lay<float, 32>::bytes_noc));
    case 64: return std::min(8, int((224 * 1024) / Lay<float, 64>::bytes_noc));
    }
    return 1;
}

cudaError_t launch_solve_batch(int np, const BatchEntry *ents, int nent, long long total, int num_sms,
                               cudaStream_t st, int warps)
{
    if (nent <= 0 || total <= 0) return cudaSuccess;
    switch (np) {
    case 16: return launch_solve_batch_t<16, true>(ents, nent, total, num_sms, st, warps);
    case 32: return launch_solve_batch_t<32, true>(ents, nent, total, num_sms, st, warps);
    case 64: return launch_solve_batch_t<64, true>(ents, nent, total, num_sms, st, warps);
    }
    return cudaErrorInvalidValue;
}

}  // namespace fpl
