// Instantiations of the fused STFT kernel for window exponents 6 7 8 9 10.
#include "stft_fused_kernel.cuh"

namespace ocs {

cudaError_t launch_fused_lo(int exp, int outk, bool staged, const FusedArgs& a, int grid, cudaStream_t st)
{
    switch (exp) {
    case 6: return launch_fused_exp<6>(outk, staged, a, grid, st);
    case 7: return launch_fused_exp<7>(outk, staged, a, grid, st);
    case 8: return launch_fused_exp<8>(outk, staged, a, grid, st);
    case 9: return launch_fused_exp<9>(outk, staged, a, grid, st);
    case 10: return launch_fused_exp<10>(outk, staged, a, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

int occupancy_lo(int exp, int outk, bool staged)
{
    switch (exp) {
    case 6: return occupancy_exp<6>(outk, staged);
    case 7: return occupancy_exp<7>(outk, staged);
    case 8: return occupancy_exp<8>(outk, staged);
    case 9: return occupancy_exp<9>(outk, staged);
    case 10: return occupancy_exp<10>(outk, staged);
    default: return 0;
    }
}

}  // namespace ocs
