// Paired-frame STFT kernel on packed FP32x2 arithmetic (window 2^10, sm_103a).
//
// The computation is that of stft_pair_kernel<10>: two consecutive real frames
// a = 2p and b = 2p+1 ride in one 1024-point complex FFT z = y_a + i y_b, the
// window table carries the factor 1/2 of the separation
//   A[k] = Z[k] + conj Z[N-k],   B[k] = (Z[k] - conj Z[N-k]) / i,
// and power or half-complex values are stored straight from registers.  Per
// frame this is the reference's Overlap_Common -> Window_* -> DCRemove_Common
// -> Stockham FFT -> toPower / toHalfComplexFormat (OKL/EXPCommon.okl:7-245,
// OKL/kernel.okl:178-218).
//
// What differs is the arithmetic: Blackwell issues add/sub/mul/fma on a pair of
// FP32 lanes as one instruction (.f32x2), which halves the issue slots the
// butterflies take, and the scalar kernel is bound by instruction issue.  The
// thread's 32 complex points live in 16 register pairs C2 {re, im}, each pair
// holding the same component of two points:
//   stage 1 (radix 32 over the frame samples t + 32u): pair j holds points
//     u = j and u = j + 16.  The first decimation-in-frequency level pairs
//     exactly those two, so it runs across the lanes in scalar code; the rest
//     is a 16-point DFT per lane, both lanes in one packed instruction stream.
//     Its outputs come out as pairs (V[2k], V[2k+1]).
//   stage 2 (radix 32 over the exchanged points t + 32u, after the twiddles
//     W_1024^{t u}): pair j holds u = 2j and u = 2j + 1.  Decimation in time:
//     a 16-point DFT per lane (even and odd u), then one level across the lanes
//     that leaves pair k = (Z[t + 32k], Z[t + 32k + 512]).
// The exchange between the stages goes through two shared-memory planes (real
// and imaginary parts) laid out so that stage 2 reads each of its pairs with
// one 8-byte load: point p = 64 r + c sits at r * 66 + 2 (c mod 32) + c / 32.
// Stage 1 writes with 4-byte stores; both sides are free of bank conflicts
// (thread t of stage 1 lands on bank t, stage 2 reads 64 consecutive words).
#pragma once
#include "ocs_x2.cuh"
#include "stft_pair_kernel.cuh"

namespace ocs {

constexpr int kPx2Exp = 10;
constexpr int kPx2Row = 66;                  // floats per row of an exchange plane (64 + 2 padding)
constexpr int kPx2Plane = 16 * kPx2Row;      // floats per plane (1024 points)
// frame pairs per CTA (one warp each); 9 warps per CTA at 108 registers (18
// warps per SM against 16) measured no faster: 447-451 against 452 Gsamples/s
constexpr int kPx2PPC = 8;
constexpr int kPx2Threads = 32 * kPx2PPC;
constexpr size_t kPx2Smem = 512 * 16         // stage-2 twiddles, float4 per (pair slot, thread)
                            + 512 * 8        // window pairs
                            + (size_t)kPx2PPC * 2 * kPx2Plane * 4;

template <int OUTK>
__global__ void __launch_bounds__(kPx2Threads, 2) stft_pairx2_kernel(const FusedArgs a)
{
    using namespace x2;
    constexpr int N = 1024, H = 512;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ float4 smem4[];
    float4* s_tw = smem4;                                   // [j * 32 + t]: W^{t 2j}, W^{t (2j+1)}
    float2* s_w = reinterpret_cast<float2*>(smem4 + 512);  // [j * 32 + t]: w[t + 32 j], w[t + 32 j + 512]
    float* planes = reinterpret_cast<float*>(s_w + 512);
    const int tid = threadIdx.x;
    const int lp = tid >> 5, t = tid & 31;
    // tables: the pair plan's stage-2 twiddles W_1024^{t m} (entry (m - 1) * 32 + t)
    // regrouped by lane pair, and the window (scaled by 1/2) regrouped likewise
    for (int i = tid; i < 512; i += blockDim.x) {
        const int jj = i >> 5, tt = i & 31;
        const float2 w0 = jj == 0 ? make_float2(1.0f, 0.0f) : a.tw[(2 * jj - 1) * 32 + tt];
        const float2 w1 = a.tw[(2 * jj) * 32 + tt];
        s_tw[i] = make_float4(w0.x, w1.x, w0.y, w1.y);
        s_w[i] = make_float2(a.win[i], a.win[i + H]);
    }
    __syncthreads();
    float* pre = planes + lp * 2 * kPx2Plane;
    float* pim = pre + kPx2Plane;
    const int src = (32 - t) & 31;
    const uint64_t pairs = (a.frames + 1) / 2;
    const uint64_t stride = (uint64_t)gridDim.x * kPx2PPC;

    for (uint64_t p = (uint64_t)blockIdx.x * kPx2PPC + lp; p < pairs; p += stride) {
        // the samples of this warp's next pair start toward L2 while this pair
        // computes (the 16-byte-aligned interior of its span, a single-GPU
        // bulk prefetch: no shared memory or registers held)
        if (t == 0 && p + stride < pairs) {
            const uint64_t s0 = 2 * (p + stride) * a.hop;
            prefetch_l2_span(a.x, s0, s0 + a.hop + N < a.n ? s0 + a.hop + N : a.n);
        }
        const uint64_t fa = 2 * p, fb = fa + 1;
        const bool act_b = fb < a.frames;  // frame a is always active here
        C2 v[16];
        // ---------------- framing + window: pair j = samples (t + 32 j, t + 32 j + 512)
        {
            const uint64_t sa = fa * a.hop, sb = sa + a.hop;
            const float* xa = a.x + sa;
            const float* xb = a.x + sb;
            if (act_b && sb + N <= a.n && a.hop == (uint64_t)H) {
                // frame b starts 512 samples after frame a: its first half is frame a's second half
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    v[j].re = make_float2(xa[t + 32 * j], xa[t + 32 * j + H]);
                    v[j].im = make_float2(v[j].re.y, xb[t + 32 * j + H]);
                }
            } else if (act_b && sb + N <= a.n && a.hop == (uint64_t)(N / 4)) {
                // overlap 0.75: frame b's sample t + 32 j is frame a's t + 32 (j + 8)
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j].re = make_float2(xa[t + 32 * j], xa[t + 32 * j + H]);
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    v[j].im = j < 8 ? v[j + 8].re : make_float2(v[j - 8].re.y, xb[t + 32 * j + H]);
            } else if (act_b && sb + N <= a.n) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    v[j].re = make_float2(xa[t + 32 * j], xa[t + 32 * j + H]);
                    v[j].im = make_float2(xb[t + 32 * j], xb[t + 32 * j + H]);
                }
            } else {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int c0 = t + 32 * j, c1 = c0 + H;
                    v[j].re = make_float2(sa + c0 < a.n ? xa[c0] : 0.0f, sa + c1 < a.n ? xa[c1] : 0.0f);
                    v[j].im = make_float2(act_b && sb + c0 < a.n ? xb[c0] : 0.0f,
                                          act_b && sb + c1 < a.n ? xb[c1] : 0.0f);
                }
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float2 w = s_w[32 * j + t];
                v[j].re = mul2(v[j].re, w);
                v[j].im = mul2(v[j].im, w);
            }
        }
        if (a.remove_dc) {
            // frame a is the real part, frame b the imaginary part
            float2 sr = v[0].re, si = v[0].im;
#pragma unroll
            for (int j = 1; j < 16; ++j) {
                sr = add2(sr, v[j].re);
                si = add2(si, v[j].im);
            }
            float s_a = sr.x + sr.y, s_b = si.x + si.y;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                s_a += __shfl_xor_sync(FULL, s_a, o);
                s_b += __shfl_xor_sync(FULL, s_b, o);
            }
            const float2 ma = bc(s_a * (1.0f / (float)N)), mb = bc(s_b * (1.0f / (float)N));
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                v[j].re = sub2(v[j].re, ma);
                v[j].im = sub2(v[j].im, mb);
            }
        }

        // ---------------- stage 1: radix-32 DFT over u of z[t + 32 u]
        static_for<0, 16>([&](auto jc) {
            constexpr int j = decltype(jc)::value;
            const float2 x0 = lane0(v[j]), x1 = lane1(v[j]);
            v[j] = pack(cadd(x0, x1), twc<j, 32>(csub(x0, x1)));
        });
        dft_lanes<16>(v);  // pair k = (V[2k], V[2k + 1])
        __syncwarp();  // the previous pair's reads of these planes are done
        {
            // V[m] goes to point 32 t + m: row t / 2, column 32 (t mod 2) + m
            const int base = (t >> 1) * kPx2Row + (t & 1);
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                pre[base + 4 * k] = v[k].re.x;
                pre[base + 4 * k + 2] = v[k].re.y;
                pim[base + 4 * k] = v[k].im.x;
                pim[base + 4 * k + 2] = v[k].im.y;
            }
        }
        __syncwarp();
        // ---------------- stage 2: pair j = points (t + 64 j, t + 64 j + 32), times W_1024^{t u}
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const float2 r = *reinterpret_cast<const float2*>(pre + j * kPx2Row + 2 * t);
            const float2 i = *reinterpret_cast<const float2*>(pim + j * kPx2Row + 2 * t);
            const float4 w = s_tw[j * 32 + t];
            const float2 wc = make_float2(w.x, w.y), ws = make_float2(w.z, w.w);
            // (r + i I)(wc + ws I) = (r wc - i ws, r ws + i wc)
            v[j].re = fma2(i, make_float2(-ws.x, -ws.y), mul2(r, wc));
            v[j].im = fma2(r, ws, mul2(i, wc));
        }
        dft_lanes<16>(v);  // pair k = (E[k], O[k]) over even and odd u
        static_for<0, 16>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            const float2 e = lane0(v[k]);
            const float2 o = twc<k, 32>(lane1(v[k]));
            v[k] = pack(cadd(e, o), csub(e, o));  // (Z[t + 32 k], Z[t + 32 k + 512])
        });

        // ---------------- separate the two spectra and store
        // bin k = t + 32 u (u < 16) is lane 0 of pair u; its partner Z[N - k] is
        // lane 1 of pair 15 - u in thread (32 - t) mod 32.  Thread 0 holds its own
        // partners (lane 1 of pair 16 - u) and also owns bin N/2 (lane 1 of pair 0).
        static_for<0, 17>([&](auto uc) {
            constexpr int u = decltype(uc)::value;
            float2 z, pz;
            if constexpr (u < 16) {
                z = lane0(v[u]);
                float2 q;
                q.x = __shfl_sync(FULL, v[15 - u].re.y, src);
                q.y = __shfl_sync(FULL, v[15 - u].im.y, src);
                if constexpr (u == 0) pz = (t == 0) ? z : q;
                else pz = (t == 0) ? lane1(v[16 - u]) : q;
            } else {
                if (t != 0) return;
                z = lane1(v[0]);
                pz = z;
            }
            const int k = t + 32 * u;
            const float2 A = make_float2(z.x + pz.x, z.y - pz.y);  // frame a, bin k
            const float2 B = make_float2(z.y + pz.y, pz.x - z.x);  // frame b, bin k
            if constexpr (OUTK == OUT_POWER || OUTK == OUT_POWER_SERIAL) {
                const float pa = power_of<OUTK>(A);
                const float pb = power_of<OUTK>(B);
                if (!a.dense) {
                    float* ra = a.out + fa * (uint64_t)N;
                    constexpr bool inner = u != 0 && u != 16;
                    const bool mirror = inner || (k != 0 && k != H);
                    if (act_b) {
                        __stcs(ra + k, pa);
                        __stcs(ra + N + k, pb);
                        if (mirror) {
                            __stcs(ra + (N - k), pa);
                            __stcs(ra + N + (N - k), pb);
                        }
                    } else {
                        __stcs(ra + k, pa);
                        if (mirror) __stcs(ra + (N - k), pa);
                    }
                } else {
                    float* ra = a.out + fa * (uint64_t)(H + 1);
                    __stcs(ra + k, pa);
                    if (act_b) __stcs(ra + (H + 1) + k, pb);
                }
            } else if constexpr (OUTK == OUT_HALF) {
                float2* o2 = reinterpret_cast<float2*>(a.out);
                if (!a.dense) {
                    const uint64_t fla = fa * (uint64_t)N;
                    const uint64_t flb = fla + N;
                    if (fla + k < a.ohalf) __stcs(o2 + fla + k, A);
                    if (k != 0 && k != H && fla + (N - k) < a.ohalf) __stcs(o2 + fla + (N - k), make_float2(A.x, -A.y));
                    if (act_b && flb + k < a.ohalf) __stcs(o2 + flb + k, B);
                    if (act_b && k != 0 && k != H && flb + (N - k) < a.ohalf)
                        __stcs(o2 + flb + (N - k), make_float2(B.x, -B.y));
                } else {
                    float2* ra = o2 + fa * (uint64_t)(H + 1);
                    __stcs(ra + k, A);
                    if (act_b) __stcs(ra + (H + 1) + k, B);
                }
            }
        });
    }
}

}  // namespace ocs
