// Instantiations of the fused STFT kernel for window exponents 11 12 13 14 15.
#include "stft_fused_kernel.cuh"

namespace ocs {

cudaError_t launch_fused_hi(int exp, int outk, bool staged, const FusedArgs& a, int grid, cudaStream_t st)
{
    switch (exp) {
    case 11: return launch_fused_exp<11>(outk, staged, a, grid, st);
    case 12: return launch_fused_exp<12>(outk, staged, a, grid, st);
    case 13: return launch_fused_exp<13>(outk, staged, a, grid, st);
    case 14: return launch_fused_exp<14>(outk, staged, a, grid, st);
    case 15: return launch_fused_exp<15>(outk, staged, a, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

int occupancy_hi(int exp, int outk, bool staged)
{
    switch (exp) {
    case 11: return occupancy_exp<11>(outk, staged);
    case 12: return occupancy_exp<12>(outk, staged);
    case 13: return occupancy_exp<13>(outk, staged);
    case 14: return occupancy_exp<14>(outk, staged);
    case 15: return occupancy_exp<15>(outk, staged);
    default: return 0;
    }
}

}  // namespace ocs
