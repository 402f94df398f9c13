// Internal interface between the C-ABI host code and the CUDA kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace ocs {

enum : int {
    OCS_MODE_POWER = 0,         // |X| (or the Serial runner's sqrt(2)|Re X|)
    OCS_MODE_HALF_COMPLEX = 1,  // interleaved (re, im)
    OCS_MODE_PLANES = 2         // separate real / imaginary planes, N bins per frame
};

struct FusedArgs {
    const float* x;        // signal (or a real plane with hop = N)
    uint64_t n;            // samples readable at x
    uint64_t hop;          // frame advance in samples
    uint64_t frames;       // frames to compute
    const float* win;      // window table (N floats) or nullptr
    const float2* tw;      // twiddle table of the plan
    float* out;            // output (or real plane)
    float* out_im;         // imaginary plane (planes mode)
    uint64_t ohalf;        // compat half-complex: number of complex outputs
    int mode;              // OCS_MODE_*
    int dense;             // N/2+1 bins per frame instead of the reference's N
    int serial_power;      // sqrt(2)|Re X| as the Serial runner returns
    int remove_dc;
};

// fused single-pass STFT (windows 2^6 .. 2^15)
cudaError_t launch_fused(int exp, bool vec2, const FusedArgs& a, int grid, cudaStream_t st);
int fused_occupancy(int exp, bool vec2);
int fused_frames_per_cta(int exp);
int fused_twiddle_count(int exp);
size_t fused_smem_bytes(int exp);
cudaError_t build_twiddles(float2* tw, int exp, cudaStream_t st);

// unfused per-stage kernels behind the runnerFunction hooks
cudaError_t launch_overlap(const float* in, uint32_t ofull, uint32_t n, uint32_t exp, uint32_t hop,
                           float* real, cudaStream_t st);
cudaError_t launch_apply_window(float* data, const float* win, uint32_t ofull, uint32_t nwin, cudaStream_t st);
cudaError_t launch_remove_dc(float* data, uint32_t ofull, uint32_t nwin, cudaStream_t st);
cudaError_t launch_half_complex(float* out, const float* re, const float* im, uint32_t ohalf, cudaStream_t st);
cudaError_t launch_to_power(float* out, const float* re, const float* im, uint32_t ofull, cudaStream_t st);

}  // namespace ocs
