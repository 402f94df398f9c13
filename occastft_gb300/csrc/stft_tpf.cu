// Thread-per-frame STFT for window 2^6 (sm_103a).
//
// At N = 64 the cooperative kernels spend most of their instructions on
// moving data between the threads that share a frame (shuffles, exchange
// buffers, barriers): a frame is only 32 complex points.  Here one lane owns
// one whole frame instead, so the FFT, the real-input untangle, DC removal and
// the power are all register arithmetic:
//   * a warp takes 32 consecutive frames; their samples arrive by cp.async in
//     32 shared-memory rows of N + 4 floats (16-byte chunks, zero-filled past
//     the signal end or the last frame);
//   * lane i reads row i with 16-byte loads (the +4 padding makes the eight
//     lanes of each quarter-warp hit disjoint banks), applies the window
//     (pre-scaled by 1/2, as in the fused kernels), removes the mean, runs a
//     32-point DFT in registers and untangles with compile-time twiddles;
//   * the N output floats go back into the same row with 16-byte stores and
//     leave as one coalesced block of 32 frames.
// Outputs: power (|X| or the Serial runner's sqrt(2)|Re X|) in the reference
// layout or the dense layout.  Half-complex stays with the cooperative kernels.
// It is the same pipeline as the fused kernels (Overlap_Common, Window_*,
// DCRemove_Common, Stockham FFT, toPower; OKL/EXPCommon.okl:7-245,
// OKL/kernel.okl:178-194).
#include "stft_fused_kernel.cuh"

namespace ocs {
namespace {

constexpr int kTpfThreads = 256;  // 8 warps, 32 frames each per step

template <int EXP>
struct TpfCfg {
    static constexpr int N = 1 << EXP;
    static constexpr int M = N / 2;
    static constexpr int RS = N + 4;  // row stride in floats (16-byte aligned, conflict-free 16-byte access)
    static constexpr size_t SMEM = (size_t)N * 4 + (size_t)(kTpfThreads / 32) * 32 * RS * 4;
};

template <int EXP, int OUTK>
__global__ void __launch_bounds__(kTpfThreads, 2) stft_tpf_kernel(const FusedArgs a)
{
    using C = TpfCfg<EXP>;
    constexpr int N = C::N, M = C::M, RS = C::RS;
    static_assert(OUTK == OUT_POWER || OUTK == OUT_POWER_SERIAL, "power outputs only");
    extern __shared__ float4 smem4[];
    float* s_win = reinterpret_cast<float*>(smem4);  // N floats, window x 1/2
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float* rows = s_win + N + warp * 32 * RS;
    for (int i = tid; i < N; i += kTpfThreads) s_win[i] = a.win[i];
    __syncthreads();

    const int cs = a.cs;  // bytes per async copy: 16, 8 or 4
    const int per_chunk = cs / 4;
    const int chunks = N / per_chunk;
    const uint64_t wstride = (uint64_t)gridDim.x * (kTpfThreads / 32);
    for (uint64_t g = (uint64_t)blockIdx.x * (kTpfThreads / 32) + warp; g * 32 < a.frames; g += wstride) {
        const uint64_t f0 = g * 32;
        // ---------------- 32 frames -> 32 rows
        if (cs == 16) {
            // N / 4 chunks per row: a lane keeps its column, rows advance by
            // 32 / (N / 4) per step, so the addresses are plain increments
            constexpr int CPR = N / 4, RSTEP = 32 / CPR;
            const int col = lane % CPR, j0 = lane / CPR;
            uint64_t f = f0 + j0;
            uint64_t pos = f * a.hop + (uint64_t)col * 4;
            const uint64_t pstep = (uint64_t)RSTEP * a.hop;
            float* dst = rows + j0 * RS + col * 4;
#pragma unroll 4
            for (int it = 0; it < 32 / RSTEP; ++it) {
                int bytes = 0;
                if (f < a.frames && pos < a.n) {
                    const uint64_t left = a.n - pos;
                    bytes = left >= 4 ? 16 : (int)left * 4;
                }
                cp_async(dst, bytes ? a.x + pos : a.x, bytes, 16);
                f += RSTEP;
                pos += pstep;
                dst += RSTEP * RS;
            }
        } else {
            for (int q = lane; q < 32 * chunks; q += 32) {
                const int jj = q / chunks, col = q - jj * chunks;
                const uint64_t f = f0 + jj;
                const uint64_t pos = f * a.hop + (uint64_t)col * per_chunk;
                int bytes = 0;
                if (f < a.frames && pos < a.n) {
                    const uint64_t left = a.n - pos;
                    bytes = left >= (uint64_t)per_chunk ? cs : (int)left * 4;
                }
                cp_async(rows + jj * RS + col * per_chunk, bytes ? a.x + pos : a.x, bytes, cs);
            }
        }
        cp_async_commit();
        cp_async_wait_all();
        __syncwarp();

        // ---------------- the lane's frame
        float2 v[M];
        const float* row = rows + lane * RS;
#pragma unroll
        for (int j = 0; j < M / 2; ++j) {
            const float4 d = *reinterpret_cast<const float4*>(row + 4 * j);
            const float4 w = *reinterpret_cast<const float4*>(s_win + 4 * j);
            v[2 * j] = make_float2(d.x * w.x, d.y * w.y);
            v[2 * j + 1] = make_float2(d.z * w.z, d.w * w.w);
        }
        if (a.remove_dc) {
            float s = 0.0f;
#pragma unroll
            for (int j = 0; j < M; ++j) s += v[j].x + v[j].y;
            // the window carries 1/2: the mean of the scaled frame is subtracted
            const float mean = s * (1.0f / (float)N);
#pragma unroll
            for (int j = 0; j < M; ++j) {
                v[j].x -= mean;
                v[j].y -= mean;
            }
        }
        dft_inreg<M, M, 0, 1>(v);  // Z[k] in slot k
        __syncwarp();              // every lane has read its row

        // ---------------- untangle, power, back into the row
        float o[OUTK == OUT_POWER || OUTK == OUT_POWER_SERIAL ? N : 1];
        static_for<0, M / 2 + 1>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            const float2 A = v[k];
            const float2 B = v[(M - k) % M];
            const float2 e = make_float2(A.x + B.x, A.y - B.y);
            const float2 od = make_float2(A.y + B.y, B.x - A.x);
            const float2 wo = twc<k, N>(od);
            const float p0 = power_of<OUTK>(make_float2(e.x + wo.x, e.y + wo.y));  // |X[k]|
            const float p1 = power_of<OUTK>(make_float2(e.x - wo.x, e.y - wo.y));  // |X[k + M]|
            o[k] = p0;
            if constexpr (k != 0) o[N - k] = p0;
            if constexpr (k != M / 2) {  // at k = M/2, k + M = N - k: keep p0
                o[k + M] = p1;
                if constexpr (k != 0) o[M - k] = p1;
            }
        });
        float* orow = rows + lane * RS;
        if (!a.dense) {
#pragma unroll
            for (int j = 0; j < N / 4; ++j)
                *reinterpret_cast<float4*>(orow + 4 * j) = make_float4(o[4 * j], o[4 * j + 1], o[4 * j + 2], o[4 * j + 3]);
        } else {
#pragma unroll
            for (int k = 0; k <= M; ++k) orow[k] = o[k];
        }
        __syncwarp();

        // ---------------- 32 rows -> HBM, coalesced
        const int nf = (a.frames - f0) < 32 ? (int)(a.frames - f0) : 32;
        if (!a.dense) {
            float4* dst = reinterpret_cast<float4*>(a.out + f0 * (uint64_t)N);
            constexpr int cpr = N / 4;
            for (int q = lane; q < nf * cpr; q += 32) {
                const int jj = q / cpr, col = q - jj * cpr;
                __stcs(dst + q, *reinterpret_cast<const float4*>(rows + jj * RS + col * 4));
            }
        } else {
            float* dst = a.out + f0 * (uint64_t)(M + 1);
            constexpr int rw = M + 1;
            for (int q = lane; q < nf * rw; q += 32) {
                const int jj = q / rw, col = q - jj * rw;
                __stcs(dst + q, rows[jj * RS + col]);
            }
        }
        __syncwarp();  // the rows take the next frames
    }
    cp_async_wait_all();
}

template <int EXP, int OUTK>
cudaError_t launch_tpf_t(const FusedArgs& a, int grid, cudaStream_t st)
{
    auto k = stft_tpf_kernel<EXP, OUTK>;
    static bool attr_set = false;
    if (!attr_set) {
        const cudaError_t e =
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TpfCfg<EXP>::SMEM);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    k<<<grid, kTpfThreads, TpfCfg<EXP>::SMEM, st>>>(a);
    return cudaGetLastError();
}

template <int EXP, int OUTK>
int occupancy_tpf_t()
{
    int blocks = 0;
    auto k = stft_tpf_kernel<EXP, OUTK>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TpfCfg<EXP>::SMEM) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k, kTpfThreads, TpfCfg<EXP>::SMEM) != cudaSuccess)
        return 0;
    return blocks;
}

}  // namespace

bool tpf_has(int exp, int outk) { return exp == 6 && (outk == OUT_POWER || outk == OUT_POWER_SERIAL); }
int tpf_frames_per_cta() { return kTpfThreads; }

cudaError_t launch_tpf(int exp, int outk, const FusedArgs& a, int grid, cudaStream_t st)
{
    if (exp != 6) return cudaErrorInvalidValue;
    if (outk == OUT_POWER) return launch_tpf_t<6, OUT_POWER>(a, grid, st);
    if (outk == OUT_POWER_SERIAL) return launch_tpf_t<6, OUT_POWER_SERIAL>(a, grid, st);
    return cudaErrorInvalidValue;
}

int tpf_occupancy(int exp, int outk)
{
    if (exp != 6) return 0;
    if (outk == OUT_POWER) return occupancy_tpf_t<6, OUT_POWER>();
    if (outk == OUT_POWER_SERIAL) return occupancy_tpf_t<6, OUT_POWER_SERIAL>();
    return 0;
}

}  // namespace ocs
