// Instantiations of the packed-FP32x2 paired-frame STFT kernel (window 2^10).
#include "stft_pairx2_kernel.cuh"

namespace ocs {

namespace {
template <int OUTK>
cudaError_t launch_px2_t(const FusedArgs& a, int grid, cudaStream_t st)
{
    const cudaError_t e = ensure_smem_attr<stft_pairx2_kernel<OUTK>>(kPx2Smem);
    if (e != cudaSuccess) return e;
    stft_pairx2_kernel<OUTK><<<grid, 256, kPx2Smem, st>>>(a);
    return cudaGetLastError();
}
template <int OUTK>
int occupancy_px2_t()
{
    int blocks = 0;
    auto k = stft_pairx2_kernel<OUTK>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPx2Smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k, 256, kPx2Smem) != cudaSuccess) return 0;
    return blocks;
}
}  // namespace

bool pairx2_has(int exp, int outk) { return exp == kPx2Exp && outk != OUT_PLANES; }
int pairx2_per_cta(int) { return kPx2PPC; }

cudaError_t launch_pairx2(int exp, int outk, const FusedArgs& a, int grid, cudaStream_t st)
{
    if (!pairx2_has(exp, outk)) return cudaErrorInvalidValue;
    switch (outk) {
    case OUT_POWER: return launch_px2_t<OUT_POWER>(a, grid, st);
    case OUT_POWER_SERIAL: return launch_px2_t<OUT_POWER_SERIAL>(a, grid, st);
    case OUT_HALF: return launch_px2_t<OUT_HALF>(a, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

int pairx2_occupancy(int exp, int outk)
{
    if (!pairx2_has(exp, outk)) return 0;
    switch (outk) {
    case OUT_POWER: return occupancy_px2_t<OUT_POWER>();
    case OUT_POWER_SERIAL: return occupancy_px2_t<OUT_POWER_SERIAL>();
    case OUT_HALF: return occupancy_px2_t<OUT_HALF>();
    default: return 0;
    }
}

}  // namespace ocs
