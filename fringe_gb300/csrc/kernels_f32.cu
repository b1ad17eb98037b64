// kernels_f32.cu -- FP32 instantiations of the pixel kernels.
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
    case 64: return launch_solve_t<64, false>(P, num_sms, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace fpl
