// Lanes-per-frame STFT body for windows 2^7 and 2^8, power outputs (sm_103a):
// L = N/64 lanes per frame, 32/L frames per warp, the FFT in registers.  Shared
// by the lanes-per-frame kernel (stft_tpf.cu) and the batch kernel's 2^8
// power tiles (stft_batch.cu).
//
// The packed M-point complex FFT (M = N/2 = 32 L) begins with one radix-L
// decimation-in-frequency step: each lane forms its own output q of that step
// from the whole row, u_q[n] = (sum_p z[n + 32p] W_L^{pq}) W_M^{nq}, n < 32, and
// its 32-point DFT in registers is then Z[Lk + q].  The untangle pairs Z[k] with
// Z[M - k] (same lane for L = 2, lanes 1 and 3 swap for L = 4) and one untangle
// gives the powers of bins k, N - k, M + k and M - k.  Frames come in by
// cp.async as padded shared rows and leave through the same rows with
// coalesced stores.  Per frame it implements the reference's Overlap_Common ->
// Window_* -> DCRemove_Common -> FFT -> toPower (OKL/EXPCommon.okl:7-245,
// OKL/kernel.okl:178-194).
#pragma once
#include "ocs_x2.cuh"
#include "stft_fused_kernel.cuh"

#include <type_traits>

namespace ocs {

// The window coefficients (scaled by 1/2) as float4s: a kernel parameter (every
// lane reads the same coefficient at a compile-time offset, which the constant
// cache serves without using the shared-memory / L1 pipe the kernels are bound
// by; N <= 256: at most 1 KB) or a copy in shared memory.
template <int N>
struct WinParam {
    float4 v[N / 4];
};
template <int N>
__device__ __forceinline__ float4 tpl_win4(const WinParam<N>& w, int i) { return w.v[i]; }
__device__ __forceinline__ float4 tpl_win4(const float4* w, int i) { return w[i]; }

// twiddle constants of the radix-L split and of the untangle, computed at
// compile time (same Taylor-series constants as the in-register DFTs)
template <int EXP>
struct TplTab {
    static constexpr int N = 1 << EXP, M = N / 2, L = N / 64;
    float tw1[2 * 32 * L];  // W_M^{n q} at [n L + q], n < 32
    float tw2[2 * 17 * L];  // W_N^{L k + q} at [k L + q], k <= 16
};

template <int EXP>
constexpr TplTab<EXP> make_tpl_tab()
{
    using T = TplTab<EXP>;
    TplTab<EXP> t{};
    for (int n = 0; n < 32; ++n)
        for (int q = 0; q < T::L; ++q) {
            const int e = (n * q) % T::M;
            t.tw1[2 * (n * T::L + q)] = (float)cx_cos(kTwoPi * e / T::M);
            t.tw1[2 * (n * T::L + q) + 1] = -(float)cx_sin(kTwoPi * e / T::M);
        }
    for (int k = 0; k <= 16; ++k)
        for (int q = 0; q < T::L; ++q) {
            const int e = (T::L * k + q) % T::N;
            t.tw2[2 * (k * T::L + q)] = (float)cx_cos(kTwoPi * e / T::N);
            t.tw2[2 * (k * T::L + q) + 1] = -(float)cx_sin(kTwoPi * e / T::N);
        }
    return t;
}

namespace {  // one copy per translation unit that runs the body
__constant__ TplTab<7> c_tpl7 = make_tpl_tab<7>();
__constant__ TplTab<8> c_tpl8 = make_tpl_tab<8>();
}  // namespace

template <int EXP>
__device__ __forceinline__ const TplTab<EXP>& tpl_tab()
{
    if constexpr (EXP == 7) return c_tpl7;
    else return c_tpl8;
}

template <int EXP>
struct TplCfg {
    static constexpr int N = 1 << EXP;
    static constexpr int M = N / 2;
    static constexpr int L = N / 64;      // lanes per frame
    static constexpr int F = 32 / L;      // frames per warp
    // input row stride: an odd number of 16-byte units, so the rows that a
    // warp's lanes read at the same column fall into distinct bank groups
    static constexpr int RS = N + 4;
    static constexpr int ORS = N + L;     // output row stride (L j + q distinct banks)
    static constexpr int THREADS = 256;   // 8 warps; two CTAs per SM (128 registers)
    static constexpr size_t SMEM = (size_t)(32 + 17) * L * 8 + (size_t)(THREADS / 32) * F * RS * 4;
    static_assert((F - 1) * ORS + N <= F * RS, "output rows fit in the input rows");
};


// the body's twiddle tables in shared memory: (32 + 17) L float2
template <int EXP>
__device__ __forceinline__ void tpl_tables(float2* s_tw1, float2* s_tw2, int tid, int nthreads)
{
    constexpr int L = TplCfg<EXP>::L;
    const TplTab<EXP>& tab = tpl_tab<EXP>();
    for (int i = tid; i < 32 * L; i += nthreads) s_tw1[i] = make_float2(tab.tw1[2 * i], tab.tw1[2 * i + 1]);
    for (int i = tid; i < 17 * L; i += nthreads) s_tw2[i] = make_float2(tab.tw2[2 * i], tab.tw2[2 * i + 1]);
}

// One warp's group g of F frames (frames g F .. g F + F - 1 below a.frames):
// rows = the warp's F input rows (reused as output rows), s_tw1 / s_tw2 the
// twiddle tables tpl_tables() fills, wp the window (scaled by 1/2) as float4s.
template <int EXP, int OUTK, typename W>
__device__ __forceinline__ void tpfl_group(const FusedArgs& a, uint64_t g, float* const rows, const float2* s_tw1,
                                           const float2* s_tw2, const W& wp, int lane)
{
    using C = TplCfg<EXP>;
    constexpr int N = C::N, M = C::M, L = C::L, F = C::F, RS = C::RS, ORS = C::ORS;
    static_assert(OUTK == OUT_POWER || OUTK == OUT_POWER_SERIAL, "power outputs only");
    static_assert(L == 2 || L == 4, "windows 2^7 and 2^8");
    const int q = lane % L, jf = lane / L;  // lane q of the warp's frame jf
    // this lane's factors: W_4^q = (cr, ci) and (-1)^q = s2 (for L = 2, (-1)^q = cr)
    const float cr = (L == 2) ? (q ? -1.0f : 1.0f) : (q == 0 ? 1.0f : q == 2 ? -1.0f : 0.0f);
    const float ci = (L == 2) ? 0.0f : (q == 1 ? -1.0f : q == 3 ? 1.0f : 0.0f);
    const float s2 = (q & 1) ? -1.0f : 1.0f;

    const int cs = a.cs;
    const int per_chunk = cs / 4;
    const int chunks = N / per_chunk;
    // group gg's F frames -> F rows at `dst_rows` (one cp.async group)
    auto load_group = [&](uint64_t gg, float* dst_rows) {
        const uint64_t f0 = gg * F;
        // the whole group inside the signal: no per-chunk bounds
        const bool full = f0 + F <= a.frames && (f0 + F - 1) * a.hop + N <= a.n;
        if (cs == 16 && full) {
            constexpr int CPR = N / 4;
            const float* src = a.x + f0 * a.hop + lane * 4;
            float* dst = dst_rows + lane * 4;
#pragma unroll 4
            for (int jj = 0; jj < F; ++jj) {
#pragma unroll
                for (int c = 0; c < CPR / 32; ++c) cp_async16(dst + jj * RS + c * 128, src + c * 128);
                src += a.hop;
            }
        } else if (cs == 16) {
            constexpr int CPR = N / 4;  // 16-byte chunks per row, a multiple of 32
            uint64_t f = f0;
            uint64_t pos0 = f0 * a.hop + (uint64_t)lane * 4;
            float* dst0 = dst_rows + lane * 4;
#pragma unroll 2
            for (int jj = 0; jj < F; ++jj) {
#pragma unroll
                for (int c = 0; c < CPR / 32; ++c) {
                    const uint64_t pos = pos0 + (uint64_t)c * 128;
                    int bytes = 0;
                    if (f < a.frames && pos < a.n) {
                        const uint64_t left = a.n - pos;
                        bytes = left >= 4 ? 16 : (int)left * 4;
                    }
                    cp_async(dst0 + c * 128, bytes ? a.x + pos : a.x, bytes, 16);
                }
                ++f;
                pos0 += a.hop;
                dst0 += RS;
            }
        } else {
            for (int t = lane; t < F * chunks; t += 32) {
                const int jj = t / chunks, col = t - jj * chunks;
                const uint64_t f = f0 + jj;
                const uint64_t pos = f * a.hop + (uint64_t)col * per_chunk;
                int bytes = 0;
                if (f < a.frames && pos < a.n) {
                    const uint64_t left = a.n - pos;
                    bytes = left >= (uint64_t)per_chunk ? cs : (int)left * 4;
                }
                cp_async(dst_rows + jj * RS + col * per_chunk, bytes ? a.x + pos : a.x, bytes, cs);
            }
        }
    };

    const uint64_t f0 = g * F;
    // (a second row set, loading the next group during this one's
    // arithmetic, measured slower: it costs a third of the warps per SM and
    // the kernel is bound by instruction issue, not by load latency)
    load_group(g, rows);
    cp_async_commit();
    cp_async_wait_all();
    __syncwarp();

    // ---------------- radix-L split of the lane's frame (the whole row)
    float2 v[32];
    const float* row = rows + jf * RS;
#pragma unroll
    for (int c = 0; c < 16; ++c) {
        float2 y0[L], y1[L];  // z[2c + 32 p], z[2c + 1 + 32 p]
#pragma unroll
        for (int p = 0; p < L; ++p) {
            const float4 d = *reinterpret_cast<const float4*>(row + 64 * p + 4 * c);
            const float4 w = tpl_win4(wp, 16 * p + c);
            y0[p] = make_float2(d.x * w.x, d.y * w.y);
            y1[p] = make_float2(d.z * w.z, d.w * w.w);
        }
        // the combinations on packed FP32x2 (both components of a complex
        // value in one instruction; each component's rounding is unchanged).
        // The window products stay scalar: from the parameter bank they take
        // the coefficient as an operand, and packed ones made the batch
        // kernel spill.
        if constexpr (L == 2) {
            // z0 + (-1)^q z1
            v[2 * c] = x2::fma2(x2::bc(cr), y0[1], y0[0]);
            v[2 * c + 1] = x2::fma2(x2::bc(cr), y1[1], y1[0]);
        } else {
            // (z0 + (-1)^q z2) + W_4^q (z1 + (-1)^q z3)
            static_for<0, 2>([&](auto hc) {
                constexpr int h = decltype(hc)::value;
                const float2* y = h ? y1 : y0;
                const float2 P = x2::fma2(x2::bc(s2), y[2], y[0]);
                const float2 Q = x2::fma2(x2::bc(s2), y[3], y[1]);
                // (cr Q.x + (-ci Q.y + P.x), cr Q.y + (ci Q.x + P.y))
                const float2 inner = x2::fma2(make_float2(-ci, ci), make_float2(Q.y, Q.x), P);
                v[2 * c + h] = x2::fma2(x2::bc(cr), Q, inner);
            });
        }
    }
    if (a.remove_dc) {
        // lane 0 of the frame summed every sample: its u_0 carries L means
        float s[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int n = 0; n < 32; ++n) s[n & 3] += v[n].x + v[n].y;
        const float corr = q == 0 ? ((s[0] + s[1]) + (s[2] + s[3])) * ((float)L / (float)N) : 0.0f;
#pragma unroll
        for (int n = 0; n < 32; ++n) {
            v[n].x -= corr;
            v[n].y -= corr;
        }
    }
#pragma unroll
    for (int n = 1; n < 32; ++n) v[n] = cmul(v[n], s_tw1[n * L + q]);
    dft_inreg<32, 32, 0, 1>(v);  // Z[L k + q] in slot k
    __syncwarp();                 // every lane has read its row

    float2 ex[L == 4 ? 16 : 1];
    if constexpr (L == 4) {
        // lanes q = 1 and 3 pair Z[4k + q] with Z[4(31 - k) + 4 - q]: the partner's slot 31 - k
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            ex[i].x = __shfl_xor_sync(0xffffffffu, v[16 + i].x, 2);
            ex[i].y = __shfl_xor_sync(0xffffffffu, v[16 + i].y, 2);
        }
    }

    // ---------------- untangle, power, into the frame's row (bins = +-q mod L)
    float* orow = rows + jf * ORS;
    float* const Pp = orow + q;
    float* const Qp = orow - q;
    static_for<0, 17>([&](auto kc) {
        constexpr int kp = decltype(kc)::value;  // k = L kp + q
        if (kp == 16 && q != 0) return;          // k = M/2 belongs to q = 0
        const float2 A = v[kp];
        float2 B;
        if constexpr (L == 2) {
            B = q ? v[(63 - kp) % 32] : v[(32 - kp) % 32];
        } else {
            const float2 b0 = v[(32 - kp) % 32], b2 = v[(63 - kp) % 32], bx = ex[(31 - kp) % 16];
            B = (q & 1) ? bx : (q ? b2 : b0);
        }
        const float2 e = make_float2(A.x + B.x, A.y - B.y);
        const float2 od = make_float2(A.y + B.y, B.x - A.x);
        const float2 wo = cmul(od, s_tw2[kp * L + q]);
        const float p0 = power_of<OUTK>(make_float2(e.x + wo.x, e.y + wo.y));  // |X[k]|
        const float p1 = power_of<OUTK>(make_float2(e.x - wo.x, e.y - wo.y));  // |X[k + M]|
        if (!a.dense) {
            Pp[L * kp] = p0;
            if (kp != 0 || q != 0) Qp[N - L * kp] = p0;
            if constexpr (kp != 16) Pp[L * kp + M] = p1;  // at k = M/2, k + M = N - k: keep p0
            if constexpr (kp != 16) {
                if (kp != 0 || q != 0) Qp[M - L * kp] = p1;
            }
        } else {
            Pp[L * kp] = p0;
            if constexpr (kp == 0) {
                if (q == 0) orow[M] = p1;  // X[M]
                else Qp[M] = p1;           // X[M - q]
            } else if constexpr (kp != 16) {
                Qp[M - L * kp] = p1;
            }
        }
    });
    __syncwarp();

    // ---------------- F rows -> HBM, coalesced
    const int nf = (a.frames - f0) < (uint64_t)F ? (int)(a.frames - f0) : F;
    if (!a.dense) {
        using V = typename std::conditional<L == 2, float2, float4>::type;
        constexpr int VPR = N / L;  // vectors per row, a multiple of 32
        V* dst = reinterpret_cast<V*>(a.out + f0 * (uint64_t)N);
        if (nf == F) {
            // t = lane + 32 i: row i / (VPR / 32), column lane + 32 (i % (VPR / 32))
            const float* srow = rows + lane * L;
            V* d = dst + lane;
#pragma unroll
            for (int i = 0; i < F * VPR / 32; ++i)
                __stcs(d + 32 * i, *reinterpret_cast<const V*>(srow + (i / (VPR / 32)) * ORS +
                                                                (i % (VPR / 32)) * 32 * L));
        } else
        for (int t = lane; t < nf * VPR; t += 32) {
            const int jj = t / VPR, col = t - jj * VPR;
            __stcs(dst + t, *reinterpret_cast<const V*>(rows + jj * ORS + col * L));
        }
    } else {
        float* dst = a.out + f0 * (uint64_t)(M + 1);
        constexpr int rw = M + 1;
        for (int t = lane; t < nf * rw; t += 32) {
            const int jj = t / rw, col = t - jj * rw;
            __stcs(dst + t, rows[jj * ORS + col]);
        }
    }
    __syncwarp();  // the rows take the next frames
}

}  // namespace ocs
