// Instantiations of the paired-frame STFT kernel for window exponents 6 7 8 9 10.
#include "stft_pair_kernel.cuh"

namespace ocs {

cudaError_t launch_pair_lo(int exp, int outk, const FusedArgs& a, int grid, cudaStream_t st)
{
    switch (exp) {
    case 6: return launch_pair_exp<6>(outk, a, grid, st);
    case 7: return launch_pair_exp<7>(outk, a, grid, st);
    case 8: return launch_pair_exp<8>(outk, a, grid, st);
    case 9: return launch_pair_exp<9>(outk, a, grid, st);
    case 10: return launch_pair_exp<10>(outk, a, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

int occupancy_pair_lo(int exp, int outk)
{
    switch (exp) {
    case 6: return occupancy_pair_exp<6>(outk);
    case 7: return occupancy_pair_exp<7>(outk);
    case 8: return occupancy_pair_exp<8>(outk);
    case 9: return occupancy_pair_exp<9>(outk);
    case 10: return occupancy_pair_exp<10>(outk);
    default: return 0;
    }
}

}  // namespace ocs
