// Fused single-pass STFT: twiddle-table builder and the dispatch over window
// exponents.  The kernel itself is stft_fused_kernel.cuh; its instantiations
// are split across stft_fused_lo.cu / stft_fused_hi.cu to compile in parallel.
#include "stft_pair_kernel.cuh"

namespace ocs {

// defined in stft_fused_lo.cu / stft_fused_hi.cu
cudaError_t launch_fused_lo(int exp, int outk, bool staged, const FusedArgs& a, int grid, cudaStream_t st);
cudaError_t launch_fused_hi(int exp, int outk, bool staged, const FusedArgs& a, int grid, cudaStream_t st);
int occupancy_lo(int exp, int outk, bool staged);
int occupancy_hi(int exp, int outk, bool staged);
cudaError_t launch_pair_lo(int exp, int outk, const FusedArgs& a, int grid, cudaStream_t st);
cudaError_t launch_pair_hi(int exp, int outk, const FusedArgs& a, int grid, cudaStream_t st);
int occupancy_pair_lo(int exp, int outk);
int occupancy_pair_hi(int exp, int outk);

// FP64 on the device, rounded once to float.
__global__ void build_twiddles_kernel(float2* tw, int exp)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const FusedCfg c = fused_cfg(exp);
    const int M = 1 << (exp - 1);
    const int size = fused_tw_size(exp);
    if (idx >= size) return;
    long long p, L;
    if (idx < M) {
        p = idx;
        L = 2LL * M;
    } else {
        int s = 1;
        while (s + 1 < c.nstages && idx >= fused_tw_offset(exp, s + 1)) ++s;
        const int e = idx - fused_tw_offset(exp, s);
        const int ns = fused_Ns(exp, s);
        const int m = e / ns + 1;
        const int j = e % ns;
        p = (long long)j * m;
        L = (long long)ns * c.radix[s];
    }
    double sn, cs;
    sincospi(2.0 * (double)(p % L) / (double)L, &sn, &cs);
    tw[idx] = make_float2((float)cs, (float)(-sn));
}

// paired-frame tables (of a plan id): stage twiddles only
__global__ void build_pair_twiddles_kernel(float2* tw, int exp)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const FusedCfg c = pair_cfg(exp);
    const int size = pair_tw_size(exp);
    if (idx >= size) return;
    long long p = 0, L = 1;
    if (c.nstages > 1) {
        int s = 1;
        while (s + 1 < c.nstages && idx >= pair_tw_offset(exp, s + 1)) ++s;
        const int e = idx - pair_tw_offset(exp, s);
        const int ns = pair_Ns(exp, s);
        const int m = e / ns + 1;
        const int j = e % ns;
        p = (long long)j * m;
        L = (long long)ns * c.radix[s];
    }
    double sn, cs;
    sincospi(2.0 * (double)(p % L) / (double)L, &sn, &cs);
    tw[idx] = make_float2((float)cs, (float)(-sn));
}

cudaError_t launch_pair(int exp, int outk, const FusedArgs& a, int grid, cudaStream_t st)
{
    if (exp >= 6 && exp <= 10) return launch_pair_lo(exp, outk, a, grid, st);
    if (exp >= 11 && exp <= 14) return launch_pair_hi(exp, outk, a, grid, st);
    return cudaErrorInvalidValue;
}

int pair_occupancy(int exp, int outk)
{
    if (exp >= 6 && exp <= 10) return occupancy_pair_lo(exp, outk);
    if (exp >= 11 && exp <= 14) return occupancy_pair_hi(exp, outk);
    return 0;
}

bool pair_has(int exp) { return pair_supported(exp); }
int pair_plan_id(int exp) { return exp == 12 ? (12 | kPairR16) : exp; }
int pair_per_cta(int exp) { return pair_ppc(pair_plan_id(exp)); }
int pair_twiddle_count(int pid) { return pair_tw_size(pid); }

cudaError_t build_pair_twiddles(float2* tw, int pid, cudaStream_t st)
{
    const int n = pair_tw_size(pid);
    build_pair_twiddles_kernel<<<(n + 255) / 256, 256, 0, st>>>(tw, pid);
    return cudaGetLastError();
}

cudaError_t launch_fused(int exp, int outk, bool staged, const FusedArgs& a, int grid, cudaStream_t st)
{
    if (exp >= 6 && exp <= 10) return launch_fused_lo(exp, outk, staged, a, grid, st);
    if (exp >= 11 && exp <= 15) return launch_fused_hi(exp, outk, staged, a, grid, st);
    return cudaErrorInvalidValue;
}

int fused_occupancy(int exp, int outk, bool staged)
{
    if (exp >= 6 && exp <= 10) return occupancy_lo(exp, outk, staged);
    if (exp >= 11 && exp <= 15) return occupancy_hi(exp, outk, staged);
    return 0;
}

bool fused_has_staged(int exp) { return exp >= 6 && fused_staged(exp); }

size_t fused_smem_bytes(int exp) { return fused_smem_bytes_ct(exp); }
int fused_frames_per_cta(int exp) { return fused_fpc(exp); }
int fused_twiddle_count(int exp) { return fused_tw_size(exp); }

cudaError_t build_twiddles(float2* tw, int exp, cudaStream_t st)
{
    const int n = fused_tw_size(exp);
    build_twiddles_kernel<<<(n + 255) / 256, 256, 0, st>>>(tw, exp);
    return cudaGetLastError();
}

}  // namespace ocs
