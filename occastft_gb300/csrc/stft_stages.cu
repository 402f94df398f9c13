// Unfused per-stage kernels behind the runnerFunction hooks
// (StandAlone/cross_gpgpu/GLOBAL/RunnerInterface.hpp:36-76).  They operate on
// the reference's [qt][N] real / imaginary planes so that a caller driving the
// stages one by one (Default_Pipeline, RunnerCommon.cpp:184-316) sees the
// reference's layout.  The FFT hook reuses the fused kernel in planes mode.
#include "ocs_kernels.h"

namespace ocs {

static inline int grid_for(uint64_t n, int threads)
{
    uint64_t g = (n + threads - 1) / threads;
    if (g > 1u << 30) g = 1u << 30;
    return (int)(g == 0 ? 1 : g);
}

// Overlap_Common (OKL/EXPCommon.okl:7-27): same 32-bit index arithmetic.
__global__ void overlap_kernel(const float* __restrict__ in, uint32_t ofull, uint32_t n, uint32_t exp,
                               uint32_t hop, float* __restrict__ real)
{
    const uint32_t mask = (1u << exp) - 1u;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ofull;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t idx = (uint32_t)i;
        const uint32_t src = (idx >> exp) * hop + (idx & mask);
        const uint32_t ex = src < n;
        real[idx] = __fmul_rn(in[src * ex], (float)ex);  // in[0] * 0 past the end, as the reference
    }
}

// Window_* (OKL/EXPCommon.okl:29-148): data[i] *= w[i mod N].
__global__ void window_kernel(float* __restrict__ data, const float* __restrict__ win, uint32_t ofull,
                              uint32_t nwin)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ofull;
         i += (uint64_t)gridDim.x * blockDim.x) {
        data[i] = data[i] * win[i & (nwin - 1)];
    }
}

// DCRemove_Common (OKL/EXPCommon.okl:151-192): one CTA per frame.
__global__ void remove_dc_kernel(float* __restrict__ data, uint32_t nwin)
{
    __shared__ float part[32];
    float* d = data + (uint64_t)blockIdx.x * nwin;
    float s = 0.0f;
    for (uint32_t i = threadIdx.x; i < nwin; i += blockDim.x) s += d[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < blockDim.x / 32 ? part[threadIdx.x] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) part[0] = s;
    }
    __syncthreads();
    const float mean = part[0] / (float)nwin;
    for (uint32_t i = threadIdx.x; i < nwin; i += blockDim.x) d[i] -= mean;
}

// toHalfComplexFormat (OKL/kernel.okl:196-218): ReadIdx == GID, a flat copy.
__global__ void half_complex_kernel(float2* __restrict__ out, const float* __restrict__ re,
                                    const float* __restrict__ im, uint32_t ohalf)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ohalf;
         i += (uint64_t)gridDim.x * blockDim.x) {
        out[i] = make_float2(re[i], im[i]);
    }
}

// toPower (OKL/kernel.okl:178-194): sqrt(R*R + I*I).
__global__ void to_power_kernel(float* __restrict__ out, const float* __restrict__ re,
                                const float* __restrict__ im, uint32_t ofull)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ofull;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const float r = re[i], m = im[i];
        out[i] = __fsqrt_rn(__fadd_rn(__fmul_rn(r, r), __fmul_rn(m, m)));
    }
}

cudaError_t launch_overlap(const float* in, uint32_t ofull, uint32_t n, uint32_t exp, uint32_t hop,
                           float* real, cudaStream_t st)
{
    overlap_kernel<<<grid_for(ofull, 256), 256, 0, st>>>(in, ofull, n, exp, hop, real);
    return cudaGetLastError();
}

cudaError_t launch_apply_window(float* data, const float* win, uint32_t ofull, uint32_t nwin, cudaStream_t st)
{
    window_kernel<<<grid_for(ofull, 256), 256, 0, st>>>(data, win, ofull, nwin);
    return cudaGetLastError();
}

cudaError_t launch_remove_dc(float* data, uint32_t ofull, uint32_t nwin, cudaStream_t st)
{
    const uint32_t frames = ofull / nwin;
    if (frames == 0) return cudaSuccess;
    const int threads = nwin >= 1024 ? 1024 : (int)nwin;
    remove_dc_kernel<<<frames, threads, 0, st>>>(data, nwin);
    return cudaGetLastError();
}

cudaError_t launch_half_complex(float* out, const float* re, const float* im, uint32_t ohalf, cudaStream_t st)
{
    half_complex_kernel<<<grid_for(ohalf, 256), 256, 0, st>>>(reinterpret_cast<float2*>(out), re, im, ohalf);
    return cudaGetLastError();
}

cudaError_t launch_to_power(float* out, const float* re, const float* im, uint32_t ofull, cudaStream_t st)
{
    to_power_kernel<<<grid_for(ofull, 256), 256, 0, st>>>(out, re, im, ofull);
    return cudaGetLastError();
}

}  // namespace ocs
