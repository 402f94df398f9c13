// Thread-per-frame STFT for windows 2^6 .. 2^8 (sm_103a).
//
// At N = 64 the cooperative kernels spend most of their instructions on
// moving data between the threads that share a frame (shuffles, exchange
// buffers, barriers): a frame is only 32 complex points.  Here one lane owns
// one whole frame instead, so the FFT, the real-input untangle, DC removal and
// the power are all register arithmetic:
//   * a warp takes 32 consecutive frames; their samples arrive by cp.async in
//     32 shared-memory rows of N + 4 floats (16-byte chunks, zero-filled past
//     the signal end or the last frame);
//   * lane i reads row i with 16-byte loads (the +4 padding puts the rows
//     that a quarter-warp reads at one column on distinct banks), applies the window
//     (pre-scaled by 1/2, as in the fused kernels), removes the mean, runs a
//     32-point DFT in registers and untangles with compile-time twiddles;
//   * the N output floats go back into the same row with 16-byte stores and
//     leave as one coalesced block of 32 frames.
// Outputs: power (|X| or the Serial runner's sqrt(2)|Re X|) in the reference
// layout or the dense layout; at N = 64 also half-complex (tpf_half_out).
//
// Windows 2^7 and 2^8 use L = N / 64 lanes per frame (stft_tpfl_kernel): the
// packed M-point complex FFT (M = N / 2 = 32 L) starts with one radix-L
// decimation-in-frequency step that every lane forms on its own from the whole
// row, keeping only its output q:
//   u_q[n] = (sum_p z[n + 32 p] W_L^{p q}) W_M^{n q},  n < 32,
// and a 32-point DFT of u_q in registers gives Z[L k + q].  The untangle pairs
// Z[k] with Z[M - k]; for L = 2 both sit in the same lane, for L = 4 lanes 1
// and 3 swap their upper 16 slots with one shuffle each.  Each lane then owns
// the bins congruent to +-q mod L and writes them into the frame's row.
// Windows 2^7 and 2^8 produce power outputs.  It is the same pipeline as the
// fused kernels (Overlap_Common, Window_*, DCRemove_Common, Stockham FFT,
// toPower / toHalfComplexFormat; OKL/EXPCommon.okl:7-245, OKL/kernel.okl:178-218).
#include "stft_tpfl_body.cuh"

#include <cstring>

namespace ocs {
namespace {

constexpr int kTpfThreads = 256;  // 8 warps, 32 frames each per step


template <int EXP>
struct TpfCfg {
    static constexpr int N = 1 << EXP;
    static constexpr int M = N / 2;
    static constexpr int RS = N + 4;  // row stride in floats (16-byte aligned, conflict-free 16-byte access)
    static constexpr size_t SMEM = (size_t)(kTpfThreads / 32) * 32 * RS * 4;
};

// Half-complex output of the lane's frame (Z[k] in v[k], k < M): the N
// complex bins leave in two passes of M, each staged in the frame's row with a
// stride of M + 1 complex values (so a half-warp's 8-byte stores hit 16
// distinct bank pairs) and copied out 32 rows at a time.  Pass 0 holds bins
// 0 .. M-1 (X[k], and X[M-k] = conj X[k+M]); pass 1 bins M .. N-1 (X[k+M], and
// X[N-k] = conj X[k]); the dense layout (bins 0 .. M) takes pass 0 plus X[M].
template <int N>
__device__ __forceinline__ void tpf_half_out(const FusedArgs& a, const float2 (&v)[N / 2], float* rows,
                                             uint64_t f0, int lane)
{
    constexpr int M = N / 2, OS = M + 1;  // output row stride in float2
    float2* rows2 = reinterpret_cast<float2*>(rows);
    float2* orow = rows2 + lane * OS;
    float2* out2 = reinterpret_cast<float2*>(a.out);
    const int nf = (a.frames - f0) < 32 ? (int)(a.frames - f0) : 32;
    static_for<0, 2>([&](auto hc) {
        constexpr int hf = decltype(hc)::value;
        if (hf == 1 && a.dense) return;
        static_for<0, M / 2 + 1>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            const float2 A = v[k];
            const float2 B = v[(M - k) % M];
            const float2 e = make_float2(A.x + B.x, A.y - B.y);
            const float2 od = make_float2(A.y + B.y, B.x - A.x);
            const float2 wo = twc<k, N>(od);
            const float2 x0 = make_float2(e.x + wo.x, e.y + wo.y);  // X[k]
            const float2 x1 = make_float2(e.x - wo.x, e.y - wo.y);  // X[k + M]
            if constexpr (hf == 0) {
                orow[k] = x0;
                if constexpr (k != 0 && k != M / 2) orow[M - k] = make_float2(x1.x, -x1.y);
                if constexpr (k == 0) {
                    if (a.dense) orow[M] = x1;
                }
            } else {
                orow[k] = x1;
                if constexpr (k != 0 && k != M / 2) orow[M - k] = make_float2(x0.x, -x0.y);
            }
        });
        __syncwarp();
        if (!a.dense) {
            // row jj, pass hf: bins hf M .. hf M + M - 1 of frame f0 + jj, flat index (f0 + jj) N + bin
            const uint64_t base = f0 * (uint64_t)N + (uint64_t)hf * M;
            if (nf == 32 && base + 31ull * N + M <= a.ohalf) {
#pragma unroll 4
                for (int jj = 0; jj < 32; ++jj)
                    for (int c = lane; c < M; c += 32) __stcs(out2 + base + (uint64_t)jj * N + c, rows2[jj * OS + c]);
            } else {
                for (int jj = 0; jj < nf; ++jj)
                    for (int c = lane; c < M; c += 32) {
                        const uint64_t flat = base + (uint64_t)jj * N + c;
                        if (flat < a.ohalf) __stcs(out2 + flat, rows2[jj * OS + c]);
                    }
            }
        } else {
            float2* dst = out2 + f0 * (uint64_t)(M + 1);
            for (int t = lane; t < nf * (M + 1); t += 32) {
                const int jj = t / (M + 1), c = t - jj * (M + 1);
                __stcs(dst + t, rows2[jj * OS + c]);
            }
        }
        __syncwarp();  // the rows take the next pass (or the next frames)
    });
}

// L2 prefetch of the sample span of frames [f0, f0 + nf) (a warp's next
// group), issued by lane 0
__device__ __forceinline__ void tpf_prefetch_group(const FusedArgs& a, uint64_t f0, int nf, int N, int lane)
{
    if (lane == 0 && f0 < a.frames) {
        const uint64_t last = f0 + (uint64_t)nf - 1 < a.frames ? f0 + (uint64_t)nf - 1 : a.frames - 1;
        const uint64_t s0 = f0 * a.hop, s1 = last * a.hop + (uint64_t)N;
        prefetch_l2_span(a.x, s0, s1 < a.n ? s1 : a.n);
    }
}

template <int EXP, int OUTK>
__global__ void __launch_bounds__(kTpfThreads, 2) stft_tpf_kernel(const FusedArgs a, const WinParam<1 << EXP> wp)
{
    using C = TpfCfg<EXP>;
    constexpr int N = C::N, M = C::M, RS = C::RS;
    static_assert(OUTK == OUT_POWER || OUTK == OUT_POWER_SERIAL || OUTK == OUT_HALF, "power or half-complex");
    extern __shared__ float4 smem4[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float* rows = reinterpret_cast<float*>(smem4) + warp * 32 * RS;

    const int cs = a.cs;  // bytes per async copy: 16, 8 or 4
    const int per_chunk = cs / 4;
    const int chunks = N / per_chunk;
    const uint64_t wstride = (uint64_t)gridDim.x * (kTpfThreads / 32);
    for (uint64_t g = (uint64_t)blockIdx.x * (kTpfThreads / 32) + warp; g * 32 < a.frames; g += wstride) {
        const uint64_t f0 = g * 32;
        tpf_prefetch_group(a, (g + wstride) * 32, 32, N, lane);
        // ---------------- 32 frames -> 32 rows
        const bool full = f0 + 32 <= a.frames && (f0 + 31) * a.hop + N <= a.n;
        if (cs == 16 && full) {
            // the whole group inside the signal: no per-chunk bounds
            constexpr int CPR = N / 4, RSTEP = 32 / CPR;
            const int col = lane % CPR, j0 = lane / CPR;
            const float* src = a.x + (f0 + j0) * a.hop + col * 4;
            const uint64_t pstep = (uint64_t)RSTEP * a.hop;
            float* dst = rows + j0 * RS + col * 4;
#pragma unroll 4
            for (int it = 0; it < 32 / RSTEP; ++it) {
                cp_async16(dst + it * RSTEP * RS, src);
                src += pstep;
            }
        } else if (cs == 16) {
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
            const float4 w = wp.v[j];
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

        if constexpr (OUTK == OUT_HALF) {
            tpf_half_out<N>(a, v, rows, f0, lane);
            continue;
        }

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
            if (nf == 32) {
                // q = lane + 32 i: row (lane / cpr) + i (32 / cpr), column lane % cpr
                constexpr int RSTEP = 32 / cpr;
                const float* srow = rows + (lane / cpr) * RS + (lane % cpr) * 4;
                float4* d = dst + lane;
#pragma unroll
                for (int i = 0; i < cpr; ++i)
                    __stcs(d + 32 * i, *reinterpret_cast<const float4*>(srow + i * RSTEP * RS));
            } else
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

template <int N>
WinParam<N> win_param(const float* host_win)
{
    WinParam<N> w;
    std::memcpy(&w, host_win, sizeof w);
    return w;
}

template <int EXP, int OUTK>
cudaError_t launch_tpf_t(const FusedArgs& a, const float* host_win, int grid, cudaStream_t st)
{
    auto k = stft_tpf_kernel<EXP, OUTK>;
    const cudaError_t e = ensure_smem_attr<stft_tpf_kernel<EXP, OUTK>>(TpfCfg<EXP>::SMEM);
    if (e != cudaSuccess) return e;
    k<<<grid, kTpfThreads, TpfCfg<EXP>::SMEM, st>>>(a, win_param<1 << EXP>(host_win));
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

// ---------------------------------------------------------------- L lanes per frame
template <int EXP, int OUTK>
__global__ void __launch_bounds__(TplCfg<EXP>::THREADS, 2) stft_tpfl_kernel(const FusedArgs a,
                                                                             const WinParam<1 << EXP> wp)
{
    using C = TplCfg<EXP>;
    constexpr int L = C::L, F = C::F, RS = C::RS, NT = C::THREADS;
    extern __shared__ float4 smem4[];
    float2* s_tw1 = reinterpret_cast<float2*>(smem4);
    float2* s_tw2 = s_tw1 + 32 * L;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float* const rows = reinterpret_cast<float*>(s_tw2 + 17 * L) + warp * F * RS;
    tpl_tables<EXP>(s_tw1, s_tw2, tid, NT);
    __syncthreads();
    const uint64_t wstride = (uint64_t)gridDim.x * (NT / 32);
    for (uint64_t g = (uint64_t)blockIdx.x * (NT / 32) + warp; g * F < a.frames; g += wstride)
        tpfl_group<EXP, OUTK>(a, g, rows, s_tw1, s_tw2, wp, lane);
    cp_async_wait_all();
}

template <int EXP, int OUTK>
cudaError_t launch_tpfl_t(const FusedArgs& a, const float* host_win, int grid, cudaStream_t st)
{
    auto k = stft_tpfl_kernel<EXP, OUTK>;
    const cudaError_t e = ensure_smem_attr<stft_tpfl_kernel<EXP, OUTK>>(TplCfg<EXP>::SMEM);
    if (e != cudaSuccess) return e;
    k<<<grid, TplCfg<EXP>::THREADS, TplCfg<EXP>::SMEM, st>>>(a, win_param<1 << EXP>(host_win));
    return cudaGetLastError();
}

template <int EXP, int OUTK>
int occupancy_tpfl_t()
{
    int blocks = 0;
    auto k = stft_tpfl_kernel<EXP, OUTK>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TplCfg<EXP>::SMEM) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k, TplCfg<EXP>::THREADS, TplCfg<EXP>::SMEM) != cudaSuccess)
        return 0;
    return blocks;
}

}  // namespace

bool tpf_has(int exp, int outk)
{
    if (outk == OUT_HALF) return exp == 6;
    return exp >= 6 && exp <= 8 && (outk == OUT_POWER || outk == OUT_POWER_SERIAL);
}
int tpf_frames_per_cta(int exp)
{
    if (exp == 7) return TplCfg<7>::THREADS / 32 * TplCfg<7>::F;
    if (exp == 8) return TplCfg<8>::THREADS / 32 * TplCfg<8>::F;
    return kTpfThreads;
}

cudaError_t launch_tpf(int exp, int outk, const FusedArgs& a, const float* host_win, int grid, cudaStream_t st)
{
    if (!host_win) return cudaErrorInvalidValue;
    const float* hw = host_win;
    if (outk == OUT_HALF) return exp == 6 ? launch_tpf_t<6, OUT_HALF>(a, hw, grid, st) : cudaErrorInvalidValue;
    const bool ser = outk == OUT_POWER_SERIAL;
    if (outk != OUT_POWER && !ser) return cudaErrorInvalidValue;
    switch (exp) {
    case 6: return ser ? launch_tpf_t<6, OUT_POWER_SERIAL>(a, hw, grid, st) : launch_tpf_t<6, OUT_POWER>(a, hw, grid, st);
    case 7:
        return ser ? launch_tpfl_t<7, OUT_POWER_SERIAL>(a, hw, grid, st) : launch_tpfl_t<7, OUT_POWER>(a, hw, grid, st);
    case 8:
        return ser ? launch_tpfl_t<8, OUT_POWER_SERIAL>(a, hw, grid, st) : launch_tpfl_t<8, OUT_POWER>(a, hw, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

int tpf_occupancy(int exp, int outk)
{
    if (outk == OUT_HALF) return exp == 6 ? occupancy_tpf_t<6, OUT_HALF>() : 0;
    const bool ser = outk == OUT_POWER_SERIAL;
    if (outk != OUT_POWER && !ser) return 0;
    switch (exp) {
    case 6: return ser ? occupancy_tpf_t<6, OUT_POWER_SERIAL>() : occupancy_tpf_t<6, OUT_POWER>();
    case 7: return ser ? occupancy_tpfl_t<7, OUT_POWER_SERIAL>() : occupancy_tpfl_t<7, OUT_POWER>();
    case 8: return ser ? occupancy_tpfl_t<8, OUT_POWER_SERIAL>() : occupancy_tpfl_t<8, OUT_POWER>();
    default: return 0;
    }
}

}  // namespace ocs
