// TEST INFRASTRUCTURE ONLY: stand-ins for the kernel interface
// (occastft_gb300/csrc/ocs_kernels.h) that the C ABI (ocs_api.cpp) drives, for
// testing its host logic without a GPU.  Each stand-in launch queues, on its
// stream, a unit of work that reads the samples of every frame it covers,
// [f*hop, f*hop + N) with zeros past the signal, as the real kernels do, and
// writes into exactly the output floats the layout gives that frame:
//   power (reference layout)     N floats per frame, float k <- sample k
//   half-complex (reference)     2N floats per frame, float k <- sample k mod N,
//                                cut at 2*OHalfSize floats in total
//   dense power / half-complex   N/2+1 or N+2 floats per frame, same rule
// so a copy that runs out of order, or a wrong offset, shows in the values.
// Size and capability queries mirror the real kernels' answers.
#include "cuda_runtime.h"
#include "fake_control.h"
#include "ocs_kernels.h"

#include <cstdint>

namespace ocs {
namespace {

void frame_out(const float* x, uint64_t n, uint64_t hop, float* out, uint64_t ohalf, bool dense, int exp, int outk,
               uint64_t f)
{
    const uint64_t N = 1ull << exp;
    const bool half = outk == OUT_HALF;
    const uint64_t row = dense ? (N / 2 + 1) * (half ? 2 : 1) : (half ? 2 * N : N);
    for (uint64_t k = 0; k < row; ++k) {
        const uint64_t idx = f * row + k;
        if (!dense && half && idx >= 2 * ohalf) break;
        const uint64_t s = f * hop + k % N;
        out[idx] = s < n ? x[s] : 0.0f;
    }
}

cudaError_t fused_like(int exp, int outk, const FusedArgs& a, cudaStream_t st)
{
    ++fake::kernel_launches;
    const FusedArgs c = a;
    fake::enqueue(st, [c, exp, outk] {
        for (uint64_t f = 0; f < c.frames; ++f) frame_out(c.x, c.n, c.hop, c.out, c.ohalf, c.dense, exp, outk, f);
    });
    return cudaSuccess;
}

cudaError_t no_work() { return cudaSuccess; }

}  // namespace

cudaError_t launch_fused(int exp, int outk, bool, const FusedArgs& a, int, cudaStream_t st)
{
    return fused_like(exp, outk, a, st);
}
int fused_occupancy(int, int, bool) { return 2; }
bool fused_has_staged(int exp) { return exp <= 9; }
int fused_frames_per_cta(int exp) { return exp <= 9 ? 8 : 2; }
int fused_twiddle_count(int exp) { return 1 << exp; }
size_t fused_smem_bytes(int) { return 0; }
cudaError_t build_twiddles(float2*, int, cudaStream_t) { return no_work(); }

bool pair_has(int exp) { return exp >= 6 && exp <= 14; }
cudaError_t launch_pair(int exp, int outk, const FusedArgs& a, int, cudaStream_t st)
{
    return fused_like(exp, outk, a, st);
}
int pair_occupancy(int, int) { return 2; }
int pair_per_cta(int) { return 4; }
int pair_plan_id(int exp) { return exp; }
int pair_twiddle_count(int pid) { return 1 << (pid & 31); }
cudaError_t build_pair_twiddles(float2*, int, cudaStream_t) { return no_work(); }

bool batch_supports(int exp) { return exp >= 6 && exp <= 13; }
int batch_tile_frames(int exp, int groups) { return (exp <= 9 ? 4 : 1) * groups; }
int batch_occupancy() { return 2; }
size_t batch_smem_bytes() { return 0; }
cudaError_t launch_batch(const FusedArgs* d_reqs, const BatchTile* d_tiles, const uint32_t* d_ntiles,
                         uint32_t* d_counter, int, cudaStream_t st)
{
    ++fake::kernel_launches;
    ++fake::launches;
    // reads the descriptors from the device copy when it runs, as the kernel does
    fake::enqueue(st, [d_reqs, d_tiles, d_ntiles, d_counter] {
        const uint32_t nt = *d_ntiles;
        for (uint32_t t = *d_counter; t < nt; ++t) {
            const BatchTile& tl = d_tiles[t];
            const FusedArgs& a = d_reqs[tl.req];
            for (uint64_t f = tl.f0; f < tl.f0 + tl.nframes; ++f)
                frame_out(a.x, a.n, a.hop, a.out, a.ohalf, a.dense, a.exp, a.outk, f);
        }
        *d_counter = nt;
    });
    return cudaSuccess;
}

bool tpf_has(int exp, int outk) { return outk == OUT_HALF ? exp == 6 : (exp >= 6 && exp <= 8); }
int tpf_frames_per_cta(int) { return 64; }
int tpf_occupancy(int, int) { return 2; }
cudaError_t launch_tpf(int exp, int outk, const FusedArgs& a, const float* host_win, int, cudaStream_t st)
{
    if (!host_win) return cudaErrorInvalidValue;
    return fused_like(exp, outk, a, st);
}

bool large_supports(int exp) { return exp >= kLargeMinExp && exp <= kLargeMaxExp; }
LargePlan large_plan(int exp)
{
    if (exp <= 22) return LargePlan{2, exp / 2, 0, exp - 1 - exp / 2};
    return LargePlan{3, 8, exp - 1 - 8 - 10, 10};
}
cudaError_t build_two_level(float2*, float2*, uint64_t, cudaStream_t) { return no_work(); }
cudaError_t launch_large(int exp, int outk, const LargeArgs& a, uint64_t frames, cudaStream_t st)
{
    ++fake::kernel_launches;
    const LargeArgs c = a;
    fake::enqueue(st, [c, exp, outk, frames] {
        for (uint64_t f = c.f0; f < c.f0 + frames && f < c.frames_total; ++f)
            frame_out(c.x, c.n, c.hop, c.out, c.ohalf, c.dense, exp, outk, f);
    });
    return cudaSuccess;
}

bool pairx2_has(int exp, int outk) { return exp == 10 && outk != OUT_PLANES; }
cudaError_t launch_pairx2(int exp, int outk, const FusedArgs& a, int, cudaStream_t st)
{
    return fused_like(exp, outk, a, st);
}
int pairx2_occupancy(int, int) { return 2; }
int pairx2_per_cta(int) { return 8; }

bool tc_supports(int exp) { return exp >= 8 && exp <= 12; }
bool tc_mode_supported(int exp, int) { return exp >= 8 && exp <= 12; }
bool tc_piped(int exp, uint64_t hop) { return (exp != 8 && exp != 10) || hop <= (1ull << exp); }
cudaError_t launch_tc(int exp, int outk, int, const FusedArgs& a, int*, int, int, cudaStream_t st)
{
    return fused_like(exp, outk, a, st);
}
cudaError_t tc_prepare(int, int) { return cudaSuccess; }

cudaError_t launch_overlap(const float*, uint32_t, uint32_t, uint32_t, uint32_t, float*, cudaStream_t)
{
    return no_work();
}
cudaError_t launch_apply_window(float*, const float*, uint32_t, uint32_t, cudaStream_t) { return no_work(); }
cudaError_t launch_remove_dc(float*, uint32_t, uint32_t, cudaStream_t) { return no_work(); }
cudaError_t launch_half_complex(float*, const float*, const float*, uint32_t, cudaStream_t) { return no_work(); }
cudaError_t launch_to_power(float*, const float*, const float*, uint32_t, cudaStream_t) { return no_work(); }

}  // namespace ocs

namespace ocs {
namespace internal {
// the no-allocation batch (a .cu file) is not part of the host stand-in build
void noalloc_forget_devices() {}
}  // namespace internal
}  // namespace ocs
