// kernels_f64.cu -- FP64 instantiations of the pixel kernels.
#include "kernels_impl.cuh"

namespace fpl {

cudaError_t launch_fp64(const KParams &P, int num_sms, cudaStream_t st)
{
    switch (pick_np(P.nb)) {
    case 16: return launch_t<double, 16>(P, num_sms, st);
    case 32: return launch_t<double, 32>(P, num_sms, st);
    case 64: return launch_t<double, 64>(P, num_sms, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace fpl
