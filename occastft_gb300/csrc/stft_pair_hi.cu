// Instantiations of the paired-frame STFT kernel for window exponents 11 12 13 14
// (at 12 the plan with 16 values per thread).
#include "stft_pair_kernel.cuh"

namespace ocs {

cudaError_t launch_pair_hi(int exp, int outk, const FusedArgs& a, int grid, cudaStream_t st)
{
    switch (exp) {
    case 11: return launch_pair_exp<11>(outk, a, grid, st);
    case 12: return launch_pair_exp<12 | kPairR16>(outk, a, grid, st);
    case 13: return launch_pair_exp<13>(outk, a, grid, st);
    case 14: return launch_pair_exp<14>(outk, a, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

int occupancy_pair_hi(int exp, int outk)
{
    switch (exp) {
    case 11: return occupancy_pair_exp<11>(outk);
    case 12: return occupancy_pair_exp<12 | kPairR16>(outk);
    case 13: return occupancy_pair_exp<13>(outk);
    case 14: return occupancy_pair_exp<14>(outk);
    default: return 0;
    }
}

}  // namespace ocs
