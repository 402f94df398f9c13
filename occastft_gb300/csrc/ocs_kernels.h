// Internal interface between the C-ABI host code and the CUDA kernels.
#pragma once
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace ocs {

// Raises Kernel's dynamic shared-memory limit to `bytes` on the current
// device, once per (kernel, device): function attributes belong to a device,
// so a runner re-initialised on another device sets them again.  Threads that
// race on the first call both set it, which is harmless.
template <auto Kernel>
inline cudaError_t ensure_smem_attr(size_t bytes)
{
    static std::atomic<uint64_t> done{0};  // bit d: device d (d < 64) is set
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev >= 0 && dev < 64 ? (1ull << dev) : 0;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_acq_rel);
    return e;
}

// output kinds of the fused kernel (compile-time specialisations)
enum : int {
    OUT_POWER = 0,         // |X|, the reference's toPower kernel
    OUT_POWER_SERIAL = 1,  // sqrt(2)|Re X|, what the reference's Serial/OpenMP runners return
    OUT_HALF = 2,          // interleaved (re, im)
    OUT_PLANES = 3,        // separate real / imaginary planes, N bins per frame
    OUT_RUNTIME = -1       // kind read from FusedArgs::outk (batch kernel)
};

struct FusedArgs {
    const float* x;        // signal (or a real plane with hop = N)
    uint64_t n;            // samples readable at x
    uint64_t hop;          // frame advance in samples
    uint64_t frames;       // frames to compute
    const float* win;      // window table scaled by 1/2 (N floats), never null
    const float2* tw;      // twiddle table of the plan
    const float2* tw_pair; // batch kernel: the two-frames-per-FFT plan's table (null: not used)
    float* out;            // output (or real plane)
    float* out_im;         // imaginary plane (planes mode)
    uint64_t ohalf;        // compat half-complex: number of complex outputs
    int dense;             // N/2+1 bins per frame instead of the reference's N
    int remove_dc;
    int vec2;              // x + f*hop is 8-byte aligned for every frame
    int cs;                // staged kernel: bytes per async copy (16, 8 or 4)
    int exp;               // window exponent (batch kernel)
    int outk;              // output kind (batch kernel)
};

// fused single-pass STFT (windows 2^6 .. 2^15)
cudaError_t launch_fused(int exp, int outk, bool staged, const FusedArgs& a, int grid, cudaStream_t st);
int fused_occupancy(int exp, int outk, bool staged);
bool fused_has_staged(int exp);
int fused_frames_per_cta(int exp);
int fused_twiddle_count(int exp);
size_t fused_smem_bytes(int exp);
cudaError_t build_twiddles(float2* tw, int exp, cudaStream_t st);

// paired-frame fused STFT (two real frames per complex FFT), windows 2^6 .. 2^14
bool pair_has(int exp);
cudaError_t launch_pair(int exp, int outk, const FusedArgs& a, int grid, cudaStream_t st);
int pair_occupancy(int exp, int outk);
int pair_per_cta(int exp);
// paired plans are named by an id: the window exponent, with a flag for the
// one-request kernel's own plan where it differs from the batch's (2^12)
int pair_plan_id(int exp);
int pair_twiddle_count(int pid);
cudaError_t build_pair_twiddles(float2* tw, int pid, cudaStream_t st);

// paired-frame STFT on packed FP32x2 arithmetic (window 2^10): same plan
// table (a.tw = the pair plan's), one warp per frame pair, 8 pairs per CTA
bool pairx2_has(int exp, int outk);
cudaError_t launch_pairx2(int exp, int outk, const FusedArgs& a, int grid, cudaStream_t st);
int pairx2_occupancy(int exp, int outk);
int pairx2_per_cta(int exp);

// uneven batch: one persistent launch over a device tile queue
struct BatchTile {
    uint32_t req;      // index into the request descriptors
    uint32_t nframes;  // frames in this tile
    uint64_t f0;       // first frame
};
bool batch_supports(int exp);
int batch_tile_frames(int exp, int groups);
int batch_occupancy();
size_t batch_smem_bytes();
cudaError_t launch_batch(const FusedArgs* d_reqs, const BatchTile* d_tiles, const uint32_t* d_ntiles,
                         uint32_t* d_counter, int grid, cudaStream_t st);

// lanes-per-frame kernels: N/64 lanes per frame, the FFT in registers
// (power at windows 2^6 .. 2^8, half-complex at 2^6)
bool tpf_has(int exp, int outk);
int tpf_frames_per_cta(int exp);
int tpf_occupancy(int exp, int outk);
// host_win: the N window coefficients a.win holds (scaled by 1/2), passed to
// the kernel as a parameter
cudaError_t launch_tpf(int exp, int outk, const FusedArgs& a, const float* host_win, int grid, cudaStream_t st);

// windows 2^16 .. 2^30: a four-step FFT of the frame's M = N/2 complex
// points.  Up to 2^22 it takes two launches (a column pass from the signal,
// M = M1 * M2, and a row pass that untangles and stores); above, three
// (M = P1 * P2 * Q: the column pass, a middle pass over P2, the row pass).
// Output kinds: power, serial power, half-complex, and planes (the stage hook).
constexpr int kLargeMinExp = 16;
constexpr int kLargeMaxExp = 30;  // OFullSize = qt * N < 2^32 leaves qt <= 3 at 2^30
struct LargePlan {
    int passes;  // 2 or 3
    int l1;      // log2 of the column FFT
    int l2;      // log2 of the middle FFT (three passes), else 0
    int l3;      // log2 of the row FFT; l1 + l2 + l3 = exp - 1
};
struct LargeArgs {
    const float* x;          // whole signal (or a real plane with hop = N)
    uint64_t n;              // its samples
    uint64_t hop;
    uint64_t f0;             // first frame of this launch (absolute)
    uint64_t frames_total;   // frames below this index are computed
    uint64_t frames_launch;  // frames of this launch (set by launch_large)
    const float* win;        // window table scaled by 1/2 (N floats); null: 1/2 throughout
    float2* scratch;         // frames of this launch x M complex
    float2* scratch2;        // the same again (three passes only)
    float* out;              // whole output (or real plane)
    float* out_im;           // imaginary plane (planes output)
    uint64_t ohalf;          // compat half-complex: complex outputs in total
    int dense;
    int remove_dc;
    uint64_t m1, m2;         // per launch: the pass's FFT length and its column (or row) count
    uint64_t col_mask;       // column pass: twiddle exponent uses column & col_mask
    const float2* tw1;       // Stockham table of the column FFT (plan of window 2^(l1+1))
    const float2* tw2;       // Stockham table of the row FFT (plan of window 2^(l3+1))
    const float2* tw3;       // Stockham table of the middle FFT (plan of window 2^(l2+1))
    const float2* twm_lo;    // exp(-2 pi i j / M): lo[j % 1024] * hi[j / 1024]
    const float2* twm_hi;
    const float2* twn_lo;    // exp(-2 pi i k / N), same split
    const float2* twn_hi;
};
bool large_supports(int exp);
LargePlan large_plan(int exp);
cudaError_t build_two_level(float2* lo, float2* hi, uint64_t L, cudaStream_t st);
cudaError_t launch_large(int exp, int outk, const LargeArgs& a, uint64_t frames, cudaStream_t st);

// tensor-core split-precision form (tcgen05), windows 2^8 .. 2^12
bool tc_supports(int exp);
// whether split mode pm exists at window 2^exp (not the bf16 hi/mid/lo split
// at 2^12, whose operands exceed shared memory)
bool tc_mode_supported(int exp, int pm);
// err: word the kernel sets to 1 when a pipeline wait gives up (after about a
// second); test_stall: test hook, the first input phase of each CTA never
// completes so that every wait runs out
// pm: operand split, 1 fp16 hi/lo, 2 bf16 hi/lo, 3 bf16 hi/mid/lo.  At 2^8
// and 2^10 the pipelined kernel needs hop <= N (tc_piped); longer frame
// advances take the first, fp16-only kernel.  2^9, 2^11 and 2^12 run the
// generic kernel, any advance.
bool tc_piped(int exp, uint64_t hop);
cudaError_t launch_tc(int exp, int outk, int pm, const FusedArgs& a, int* err, int test_stall, int sms,
                      cudaStream_t st);
// builds the DFT-matrix and twiddle tables the form (exp, pm) uses, once per
// device, so that a later launch (possibly under stream capture) finds them
cudaError_t tc_prepare(int exp, int pm);

// unfused per-stage kernels behind the runnerFunction hooks
cudaError_t launch_overlap(const float* in, uint32_t ofull, uint32_t n, uint32_t exp, uint32_t hop,
                           float* real, cudaStream_t st);
cudaError_t launch_apply_window(float* data, const float* win, uint32_t ofull, uint32_t nwin, cudaStream_t st);
cudaError_t launch_remove_dc(float* data, uint32_t ofull, uint32_t nwin, cudaStream_t st);
cudaError_t launch_half_complex(float* out, const float* re, const float* im, uint32_t ohalf, cudaStream_t st);
cudaError_t launch_to_power(float* out, const float* re, const float* im, uint32_t ofull, cudaStream_t st);

}  // namespace ocs
