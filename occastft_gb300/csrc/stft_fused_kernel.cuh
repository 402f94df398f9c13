// Fused single-pass STFT kernels (windows 2^6 .. 2^15, sm_103a).
//
// One launch does, per frame f of the signal:
//   framing  (Overlap_Common,  OKL/EXPCommon.okl:7-27)      x[f*hop + i], 0 past the end
//   window   (Window_*,        OKL/EXPCommon.okl:29-148)    * w[i] (host-generated table)
//   DC       (DCRemove_Common, OKL/EXPCommon.okl:151-192)   - mean of the windowed frame
//   FFT      (Stockhoptimized6..11 / StockHamCommon)        N-point DFT of the real frame
//   output   (toPower / toHalfComplexFormat, OKL/kernel.okl:178-218)
// reading the signal once from HBM and writing the output once; no
// intermediate frame buffers exist in global memory.
//
// Thread mapping: a frame group of T = M/R threads owns one frame; thread t
// holds complex slots u = 0..R-1, i.e. z[t + u*T] = (y[2(t+uT)], y[2(t+uT)+1]).
//
// Two I/O schemes share the FFT core:
//   direct  (stft_fused_kernel)   each frame group loads / stores its own frame
//           straight from / to HBM.  Coalesced when a frame spans >= 16 lanes.
//   staged  (stft_staged_kernel)  for small windows, where one warp holds many
//           frames: a tile of frames is copied HBM -> shared memory with 16-byte
//           cp.async into padded rows (zero-filled past the signal end), and
//           results leave through padded shared rows with 16-byte coalesced
//           stores, so every global access is a full-width transaction.
//
// The window table the kernels receive is pre-scaled by 1/2 (exact), which
// absorbs the 1/2 of the real-input untangle: with z' = z/2,
//   X[k] = (Z'[k] + conj Z'[M-k]) + W_N^k (Z'[k] - conj Z'[M-k]) / i.
#pragma once
#include "ocs_fft_core.cuh"
#include "ocs_kernels.h"

#include <type_traits>

namespace ocs {

template <int I, int N, typename F>
__device__ __forceinline__ void static_for(F&& f)
{
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        static_for<I + 1, N>(f);
    }
}

// one padding slot every 2^L slots: 2^L = R keeps both the radix-R stage
// writes (stride R) and the strided reads (stride T) free of bank conflicts
template <int L>
__device__ __forceinline__ int padl(int i) { return i + (i >> L); }
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

template <int T>
__device__ __forceinline__ void group_sync()
{
    if constexpr (T <= 32) {
        __syncwarp();
    } else {
        __syncthreads();
    }
}

__device__ __forceinline__ float fast_sqrt(float x)
{
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

template <int OUTK>
__device__ __forceinline__ float power_of(float2 x)
{
    if constexpr (OUTK == OUT_POWER_SERIAL) {
        // the Serial runner's toPower(out, Real, Real): sqrt(2 Re^2) = sqrt(2) |Re|
        return fabsf(x.x) * 1.41421356237309505f;
    } else {
        return fast_sqrt(fmaf(x.x, x.x, x.y * x.y));
    }
}

// ------------------------------------------------------------ async copies
__device__ __forceinline__ void cp_async(void* sdst, const void* gsrc, int bytes, int cs)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
    if (cs == 16) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gsrc), "r"(bytes) : "memory");
    } else if (cs == 8) {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gsrc), "r"(bytes) : "memory");
    } else {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gsrc), "r"(bytes) : "memory");
    }
}
// a whole 16-byte chunk, no bounds (the caller checked the span)
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Starts an L2 fill of samples [s0, s1) of x: the 16-byte-aligned interior of
// the span as one bulk prefetch (a hint on this GPU's own memory; it holds no
// registers or shared memory and completes on its own).  The persistent
// kernels issue it for a frame (or pair) of their next iteration, so that the
// loads of that iteration hit L2 instead of waiting on DRAM.
__device__ __forceinline__ void prefetch_l2_span(const float* x, uint64_t s0, uint64_t s1)
{
    const uintptr_t b = (reinterpret_cast<uintptr_t>(x + s0) + 15) & ~(uintptr_t)15;
    const uintptr_t e = reinterpret_cast<uintptr_t>(x + s1) & ~(uintptr_t)15;
    if (s0 < s1 && b < e)
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(b), "r"((unsigned)(e - b)) : "memory");
}

// ------------------------------------------------------------ plan constants
// tables live in shared memory up to this exponent
__host__ __device__ constexpr bool fused_tables_in_smem(int exp) { return exp <= 12; }
// staged I/O is used up to this exponent (frames narrower than 16 lanes)
__host__ __device__ constexpr bool fused_staged(int exp) { return exp <= 9; }
// padded row strides (floats) of the staged kernel
__host__ __device__ constexpr int staged_in_stride(int exp) { return (1 << exp) + 4; }
__host__ __device__ constexpr int staged_out_stride(int exp, int outk)
{
    return (outk == OUT_HALF ? 2 * (1 << exp) : (1 << exp)) + 4;
}

// Above that exponent the plan table (~8 x 2^exp bytes) does not fit next to
// the exchange buffers; the kernels then rebuild every twiddle from a
// two-level table in shared memory: W_N^e = lo[e % 128] * hi[e / 128].
__host__ __device__ constexpr size_t fused_tw2_entries(int exp) { return 128 + ((size_t)1 << exp) / 128; }
__host__ __device__ constexpr size_t fused_tab_bytes(int exp)
{
    return fused_tables_in_smem(exp) ? (size_t)fused_tw_size(exp) * 8 + (size_t)fused_M(exp) * 8
                                     : fused_tw2_entries(exp) * 8;
}

struct TwTwoLevel {
    const float2* lo;  // W_N^e, e < 128
    const float2* hi;  // W_N^(128 h), h < N / 128
};
// twiddle W_N^e that the plan table holds at index idx
__device__ __forceinline__ float2 tw_get(const float2* tw, int idx, int /*e*/) { return tw[idx]; }
__device__ __forceinline__ float2 tw_get(const TwTwoLevel& tw, int /*idx*/, int e)
{
    return cmul(tw.lo[e & 127], tw.hi[e >> 7]);
}
// Fills the two-level table from the plan table, whose first M entries are
// W_N^k (k < M); W_N^(k + M) = -W_N^k.
template <int EXP>
__device__ __forceinline__ TwTwoLevel build_tw2(const float2* plan, float2* s, int tid, int nthreads)
{
    constexpr int M = fused_M(EXP), NH = (1 << EXP) / 128;
    for (int i = tid; i < 128 + NH; i += nthreads) {
        float2 w;
        if (i < 128) {
            w = plan[i];
        } else {
            const int e = 128 * (i - 128);
            w = e < M ? plan[e] : make_float2(-plan[e - M].x, -plan[e - M].y);
        }
        s[i] = w;
    }
    return TwTwoLevel{s, s + 128};
}

__host__ __device__ constexpr size_t fused_smem_bytes_ct(int exp)
{
    return (size_t)fused_fpc(exp) * fused_buf_stride(exp) * 8 + fused_tab_bytes(exp) +
           (size_t)(fused_cta_threads(exp) / 32) * 4 + 16;
}

__host__ __device__ constexpr size_t staged_xbuf_floats(int exp, int outk)
{
    // exchange buffers double as output staging rows
    return (size_t)fused_fpc(exp) * ((size_t)fused_buf_stride(exp) * 2 > (size_t)staged_out_stride(exp, outk)
                                         ? (size_t)fused_buf_stride(exp) * 2
                                         : (size_t)staged_out_stride(exp, outk));
}

__host__ __device__ constexpr size_t staged_smem_bytes_ct(int exp, int outk)
{
    return (size_t)fused_fpc(exp) * staged_in_stride(exp) * 4 + staged_xbuf_floats(exp, outk) * 4 +
           fused_tab_bytes(exp) + (size_t)(fused_cta_threads(exp) / 32) * 4 + 16;
}

// ------------------------------------------------------------ FFT core
template <int EXP>
struct Core {
    static constexpr FusedCfg C = fused_cfg(EXP);
    static constexpr int N = 1 << EXP;
    static constexpr int M = N / 2;
    static constexpr int R = C.R;
    static constexpr int T = M / R;
    static constexpr int NS = C.nstages;
    static constexpr int LP = ilog2(R);
    static constexpr unsigned FULL = 0xffffffffu;
    static __device__ __forceinline__ int pd(int i) { return padl<LP>(i); }

    // subtract the windowed frame's mean (DCRemove_Common semantics)
    static __device__ __forceinline__ void remove_dc(float2 (&v)[R], float* red, int tid, int lf)
    {
        float sum = 0.0f;
#pragma unroll
        for (int u = 0; u < R; ++u) sum += v[u].x + v[u].y;
        if constexpr (T <= 32) {
#pragma unroll
            for (int o = T / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(FULL, sum, o);
        } else {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(FULL, sum, o);
            constexpr int WPF = T / 32;  // warps per frame
            if ((tid & 31) == 0) red[tid >> 5] = sum;
            __syncthreads();
            sum = 0.0f;
#pragma unroll
            for (int w = 0; w < WPF; ++w) sum += red[lf * WPF + w];
            __syncthreads();
        }
        const float mean = sum * (1.0f / (float)N);
#pragma unroll
        for (int u = 0; u < R; ++u) {
            v[u].x -= mean;
            v[u].y -= mean;
        }
    }

    // all Stockham stages; the last stage leaves Z[t + u*T] in slot u.
    // TW: the plan table (const float2*) or a TwTwoLevel
    template <typename TW>
    static __device__ __forceinline__ void fft(float2 (&v)[R], float2* buf, const TW& tw, int t)
    {
        {
            constexpr int r = C.radix[0];
            static_for<0, R / r>([&](auto qc) {
                constexpr int q = decltype(qc)::value;
                dft_inreg<R, r, q, R / r>(v);
            });
        }
        static_for<1, NS>([&](auto sc) {
            constexpr int s = decltype(sc)::value;
            constexpr int rp = C.radix[s - 1];  // previous stage radix
            constexpr int nsp = fused_Ns(EXP, s - 1);
            constexpr int r = C.radix[s];
            constexpr int ns = fused_Ns(EXP, s);
            constexpr int toff = fused_tw_offset(EXP, s);
            constexpr int ef = N / (ns * r);  // W_{ns r}^{j m} = W_N^{j m ef}
            group_sync<T>();
            // write the previous stage's outputs at their Stockham positions
            static_for<0, R / rp>([&](auto qc) {
                constexpr int q = decltype(qc)::value;
                const int g = t + q * T;
                const int base = (g / nsp) * nsp * rp + (g % nsp);
                static_for<0, rp>([&](auto mc) {
                    constexpr int m = decltype(mc)::value;
                    buf[pd(base + m * nsp)] = v[q + m * (R / rp)];
                });
            });
            group_sync<T>();
#pragma unroll
            for (int u = 0; u < R; ++u) v[u] = buf[pd(t + u * T)];
            // twiddle and radix-r DFT
            static_for<0, R / r>([&](auto qc) {
                constexpr int q = decltype(qc)::value;
                const int j = (t + q * T) % ns;
                if constexpr (std::is_same<TW, TwTwoLevel>::value) {
                    // W^{j m ef} for m = 1, 2, ...: a two-level lookup every
                    // 8th m and products with W^{j ef} in between (at most 7
                    // rounding steps).  The lanes' lookups stride the lo table
                    // by multiples of m ef, so each one costs several bank
                    // wavefronts; this keeps one in eight.
                    float2 b = make_float2(1.0f, 0.0f), w = b;
                    static_for<1, r>([&](auto mc) {
                        constexpr int m = decltype(mc)::value;
                        if constexpr ((m - 1) % 8 == 0) {
                            w = tw_get(tw, 0, j * m * ef);
                            if constexpr (m == 1) b = w;
                        } else {
                            w = cmul(w, b);
                        }
                        v[q + m * (R / r)] = cmul(v[q + m * (R / r)], w);
                    });
                } else {
                    static_for<1, r>([&](auto mc) {
                        constexpr int m = decltype(mc)::value;
                        v[q + m * (R / r)] = cmul(v[q + m * (R / r)], tw_get(tw, toff + (m - 1) * ns + j, j * m * ef));
                    });
                }
                dft_inreg<R, r, q, R / r>(v);
            });
        });
    }

    // Partner values Z[M - (t + u*T)].  Frames inside one warp exchange by
    // shuffle slot by slot (partner_at); wider frames go through shared memory
    // (partners_prepare once, then partner_at).
    static __device__ __forceinline__ void partners_prepare(const float2 (&v)[R], float2* buf, int t)
    {
        if constexpr (T > 32) {
            group_sync<T>();
#pragma unroll
            for (int u = 0; u < R; ++u) buf[pd(t + u * T)] = v[u];
            group_sync<T>();
        }
    }
    template <int U>
    static __device__ __forceinline__ float2 partner_at(const float2 (&v)[R], const float2* buf, int t, int src)
    {
        if constexpr (T <= 32) {
            float2 p;
            p.x = __shfl_sync(FULL, v[R - 1 - U].x, src);
            p.y = __shfl_sync(FULL, v[R - 1 - U].y, src);
            return (t == 0) ? v[(R - U) % R] : p;
        } else {
            const float2 p = buf[pd((T - t) + (R - 1 - U) * T)];
            return (t == 0) ? v[(R - U) % R] : p;
        }
    }
    static __device__ __forceinline__ int partner_lane(int tid, int t)
    {
        const int lane = tid & 31;
        return (lane & ~(T - 1)) | ((T - t) & (T - 1));
    }

    // X[k] = e + wo, X[k + M] = e - wo for k = t + u*T
    static __device__ __forceinline__ void untangle(float2 A, float2 B, float2 w, float2& e, float2& wo)
    {
        e = make_float2(A.x + B.x, A.y - B.y);
        const float2 o = make_float2(A.y + B.y, B.x - A.x);
        wo = make_float2(w.x * o.x - w.y * o.y, w.x * o.y + w.y * o.x);
    }
};

template <int EXP>
__device__ __forceinline__ void load_tables(const FusedArgs& a, float2* s_tab, int tid, const float2*& tw,
                                            const float2*& win2)
{
    constexpr int TWN = fused_tw_size(EXP);
    constexpr int M = fused_M(EXP);
    if constexpr (fused_tables_in_smem(EXP)) {
        for (int i = tid; i < TWN; i += blockDim.x) s_tab[i] = a.tw[i];
        const float2* gw = reinterpret_cast<const float2*>(a.win);
        for (int i = tid; i < M; i += blockDim.x) s_tab[TWN + i] = gw[i];
        __syncthreads();
        tw = s_tab;
        win2 = s_tab + TWN;
    } else {
        tw = a.tw;
        win2 = reinterpret_cast<const float2*>(a.win);
    }
}

// ============================================================ direct I/O kernel
// One CTA-iteration: frames [fbase + lf] for every frame group of the CTA.
// OUTK may be OUT_RUNTIME, in which case a.outk selects the output kind
// (the batch kernel mixes requests of different kinds).
template <int EXP, int OUTK, typename TW = const float2*>
__device__ __forceinline__ void fused_group_frames(const FusedArgs& a, uint64_t fbase, float2* buf, float* red,
                                                   const TW& tw, const float2* win2, int tid, int lf, int t)
{
    using K = Core<EXP>;
    constexpr int N = K::N, M = K::M, R = K::R, T = K::T;
    const bool vec2 = a.vec2 != 0;
    const int outk = OUTK == OUT_RUNTIME ? a.outk : OUTK;
    const uint64_t f = fbase + lf;
    const bool active = f < a.frames;
    float2 v[R];

    // ---------------- framing + window (one HBM read of the frame)
    {
        const uint64_t s = f * a.hop;
        const float* xs = a.x + s;
        if (active && s + N <= a.n) {
            if (vec2) {
#pragma unroll
                for (int u = 0; u < R; ++u) v[u] = reinterpret_cast<const float2*>(xs)[t + u * T];
            } else {
#pragma unroll
                for (int u = 0; u < R; ++u) {
                    const int c = t + u * T;
                    v[u] = make_float2(xs[2 * c], xs[2 * c + 1]);
                }
            }
        } else if (active) {
#pragma unroll
            for (int u = 0; u < R; ++u) {
                const uint64_t c = (uint64_t)(t + u * T);
                const uint64_t i0 = s + 2 * c;
                v[u] = make_float2(i0 < a.n ? xs[2 * c] : 0.0f, i0 + 1 < a.n ? xs[2 * c + 1] : 0.0f);
            }
        } else {
#pragma unroll
            for (int u = 0; u < R; ++u) v[u] = make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int u = 0; u < R; ++u) {
            const float2 w = win2[t + u * T];
            v[u].x *= w.x;
            v[u].y *= w.y;
        }
    }
    if (a.remove_dc) K::remove_dc(v, red, tid, lf);
    K::fft(v, buf, tw, t);
    K::partners_prepare(v, buf, t);
    const int src = K::partner_lane(tid, t);

    // ---------------- untangle + fused output store
    // Power and planes: one untangle at bin k < M/2 gives X[k] and X[k + M],
    // and with them, for a real frame, X[N - k] = conj X[k] and
    // X[M - k] = conj X[M + k], so slots u < R/2 (k = t + u T < M/2) cover
    // every bin and slot R/2 of the group's first thread adds k = M/2.
    // Half-complex keeps one untangle per slot: its mirrored 8-byte stores
    // would start off the 64-byte boundaries its direct stores keep (measured
    // slower, 2^7 0.85 -> 0.66 of HBM), so it writes X[k] and X[k + M] only.
    constexpr bool HALF_ONLY = OUTK == OUT_HALF;
    constexpr bool NO_HALF = OUTK == OUT_POWER || OUTK == OUT_POWER_SERIAL || OUTK == OUT_PLANES;
    static_for<0, NO_HALF ? R / 2 + 1 : R>([&](auto uc) {
        constexpr int u = decltype(uc)::value;
        const float2 pu = K::template partner_at<u>(v, buf, t, src);
        if (!active) return;
        const bool half = HALF_ONLY || (!NO_HALF && outk == OUT_HALF);
        if (!half) {
            if (u > R / 2 || (u == R / 2 && t != 0)) return;
        }
        const int k = t + u * T;
        float2 e, wo;
        K::untangle(v[u], pu, tw_get(tw, k, k), e, wo);
        const float2 xa = cadd(e, wo);  // X[k]
        const float2 xb = csub(e, wo);  // X[k + M]
        const bool mid = u == R / 2;     // k = M/2 (power): X[k + M] = X[N - k]
        if (outk == OUT_POWER || outk == OUT_POWER_SERIAL) {
            const bool ser = OUTK == OUT_POWER_SERIAL || (OUTK == OUT_RUNTIME && outk == OUT_POWER_SERIAL);
            const float pa = ser ? power_of<OUT_POWER_SERIAL>(xa) : power_of<OUT_POWER>(xa);
            if (!a.dense) {
                float* row = a.out + f * (uint64_t)N;
                __stcs(row + k, pa);
                if (k != 0) __stcs(row + (N - k), pa);  // |X[N-k]| = |X[k]|
                if (!mid) {
                    const float pb = ser ? power_of<OUT_POWER_SERIAL>(xb) : power_of<OUT_POWER>(xb);
                    __stcs(row + (M + k), pb);
                    if (k != 0) __stcs(row + (M - k), pb);  // |X[M-k]| = |X[M+k]|
                }
            } else {
                float* row = a.out + f * (uint64_t)(M + 1);
                __stcs(row + k, pa);
                if (!mid) __stcs(row + (M - k), ser ? power_of<OUT_POWER_SERIAL>(xb) : power_of<OUT_POWER>(xb));
            }
        } else if (outk == OUT_HALF) {
            float2* o2 = reinterpret_cast<float2*>(a.out);
            if (!a.dense) {
                const uint64_t flat = f * (uint64_t)N + k;
                if (flat < a.ohalf) __stcs(o2 + flat, xa);
                if (flat + M < a.ohalf) __stcs(o2 + flat + M, xb);
            } else {
                float2* row = o2 + f * (uint64_t)(M + 1);
                __stcs(row + k, xa);
                if (k == 0) __stcs(row + M, xb);
            }
        } else {  // planes
            const uint64_t b = f * (uint64_t)N;
            a.out[b + k] = xa.x;
            a.out_im[b + k] = xa.y;
            a.out[b + k + M] = xb.x;
            a.out_im[b + k + M] = xb.y;
            if (!mid && k != 0) {
                a.out[b + (N - k)] = xa.x;
                a.out_im[b + (N - k)] = -xa.y;
                a.out[b + (M - k)] = xb.x;
                a.out_im[b + (M - k)] = -xb.y;
            }
        }
    });
}

// L2 prefetch of frame f (the frame this thread's group takes next), issued
// by the group's first thread
template <int EXP>
__device__ __forceinline__ void fused_prefetch_next(const FusedArgs& a, uint64_t f, int t)
{
    if (t == 0 && f < a.frames) {
        const uint64_t s0 = f * a.hop;
        const uint64_t s1 = s0 + (uint64_t)(1 << EXP) < a.n ? s0 + (uint64_t)(1 << EXP) : a.n;
        prefetch_l2_span(a.x, s0, s1);
    }
}

// CTAs per SM the register budget is sized for: three at window 2^13 (one
// frame of 256 threads, 80 registers; measured 355 -> 403 Gsamples/s for
// half-complex at 1e8 samples), otherwise two 256-thread CTAs or one larger
__host__ __device__ constexpr int fused_min_blocks(int exp)
{
    return exp == 13 ? 3 : (fused_cta_threads(exp) >= 512 ? 1 : 512 / fused_cta_threads(exp));
}

template <int EXP, int OUTK>
__global__ void __launch_bounds__(fused_cta_threads(EXP), fused_min_blocks(EXP))
stft_fused_kernel(const FusedArgs a)
{
    using K = Core<EXP>;
    constexpr int T = K::T;
    constexpr int FPC = fused_fpc(EXP);
    constexpr int BS = fused_buf_stride(EXP);

    extern __shared__ float2 smem[];
    const int tid = threadIdx.x;
    const int lf = tid / T;
    const int t = tid - lf * T;
    float2* buf = smem + lf * BS;
    float2* s_tab = smem + FPC * BS;
    float* red = reinterpret_cast<float*>(reinterpret_cast<char*>(s_tab) + fused_tab_bytes(EXP));
    if constexpr (fused_tables_in_smem(EXP)) {
        const float2* tw;
        const float2* win2;
        load_tables<EXP>(a, s_tab, tid, tw, win2);
        for (uint64_t fbase = (uint64_t)blockIdx.x * FPC; fbase < a.frames; fbase += (uint64_t)gridDim.x * FPC) {
            fused_prefetch_next<EXP>(a, fbase + (uint64_t)gridDim.x * FPC + lf, t);
            fused_group_frames<EXP, OUTK>(a, fbase, buf, red, tw, win2, tid, lf, t);
        }
    } else {
        const TwTwoLevel tw = build_tw2<EXP>(a.tw, s_tab, tid, blockDim.x);
        __syncthreads();
        const float2* win2 = reinterpret_cast<const float2*>(a.win);
        for (uint64_t fbase = (uint64_t)blockIdx.x * FPC; fbase < a.frames; fbase += (uint64_t)gridDim.x * FPC) {
            fused_prefetch_next<EXP>(a, fbase + (uint64_t)gridDim.x * FPC + lf, t);
            fused_group_frames<EXP, OUTK>(a, fbase, buf, red, tw, win2, tid, lf, t);
        }
    }
}

// ============================================================ staged I/O kernel
// Frame tile [f0, f0 + FPC): input rows of N floats (stride N + 4) are filled
// by cp.async while the previous tile computes; outputs are assembled in
// padded rows and written with 16-byte stores (compat layouts) or 4-byte
// stores of the contiguous tile (dense layouts).  Requires out 16-byte aligned.
template <int EXP, int OUTK>
__global__ void __launch_bounds__(fused_cta_threads(EXP), (fused_cta_threads(EXP) >= 512 ? 1 : 512 / fused_cta_threads(EXP)))
stft_staged_kernel(const FusedArgs a)
{
    using K = Core<EXP>;
    constexpr int N = K::N, M = K::M, R = K::R, T = K::T;
    constexpr int FPC = fused_fpc(EXP);
    constexpr int BS = fused_buf_stride(EXP);
    constexpr int IS = staged_in_stride(EXP);
    constexpr int OS = staged_out_stride(EXP, OUTK);
    constexpr int NT = fused_cta_threads(EXP);
    static_assert(OUTK != OUT_PLANES, "planes use the direct kernel");

    extern __shared__ float4 smem4[];
    float* s_in = reinterpret_cast<float*>(smem4);
    float* s_x = s_in + (size_t)FPC * IS;  // exchange buffers / output rows
    float2* s_tab = reinterpret_cast<float2*>(s_x + staged_xbuf_floats(EXP, OUTK));
    float* red = reinterpret_cast<float*>(reinterpret_cast<char*>(s_tab) + fused_tab_bytes(EXP));

    const int tid = threadIdx.x;
    const int lf = tid / T;
    const int t = tid - lf * T;
    float2* buf = reinterpret_cast<float2*>(s_x) + lf * BS;
    const float2* tw;
    const float2* win2;
    load_tables<EXP>(a, s_tab, tid, tw, win2);
    const int cs = a.cs;  // bytes per async copy: 16, 8 or 4
    const int per_chunk = cs / 4;
    constexpr int rows_chunks16 = N / 4;

    // issue the async copies of tile [f0, f0 + FPC)
    auto prefetch = [&](uint64_t f0) {
        if (cs == 16) {
            // N / 4 chunks per row, a compile-time count: no division per copy
            constexpr int CPR = N / 4;
            for (int q = tid; q < FPC * CPR; q += NT) {
                const int jj = q / CPR;
                const int col = q - jj * CPR;
                const uint64_t f = f0 + jj;
                const uint64_t pos = f * a.hop + (uint64_t)col * 4;
                int bytes = 0;
                if (f < a.frames && pos < a.n) {
                    const uint64_t left = a.n - pos;
                    bytes = left >= 4 ? 16 : (int)left * 4;
                }
                cp_async(s_in + jj * IS + col * 4, bytes ? a.x + pos : a.x, bytes, 16);
            }
            cp_async_commit();
            return;
        }
        const int chunks = N / per_chunk;
        for (int q = tid; q < FPC * chunks; q += NT) {
            const int jj = q / chunks;
            const int col = q - jj * chunks;
            const uint64_t f = f0 + jj;
            const uint64_t pos = f * a.hop + (uint64_t)col * per_chunk;
            int bytes = 0;
            if (f < a.frames && pos < a.n) {
                const uint64_t left = a.n - pos;
                bytes = left >= (uint64_t)per_chunk ? cs : (int)left * 4;
            }
            const float* src = bytes ? a.x + pos : a.x;
            cp_async(s_in + jj * IS + col * per_chunk, src, bytes, cs);
        }
        cp_async_commit();
    };

    const uint64_t stride = (uint64_t)gridDim.x * FPC;
    uint64_t fbase = (uint64_t)blockIdx.x * FPC;
    if (fbase < a.frames) prefetch(fbase);
    for (; fbase < a.frames; fbase += stride) {
        const uint64_t f = fbase + lf;
        const bool active = f < a.frames;
        float2 v[R];
        cp_async_wait_all();
        __syncthreads();
        {
            const float* row = s_in + lf * IS;
#pragma unroll
            for (int u = 0; u < R; ++u) {
                const int c = t + u * T;
                const float2 d = *reinterpret_cast<const float2*>(row + 2 * c);
                const float2 w = win2[c];
                v[u] = make_float2(d.x * w.x, d.y * w.y);
            }
        }
        __syncthreads();  // the input rows are free: fetch the next tile behind the FFT
        if (fbase + stride < a.frames) prefetch(fbase + stride);

        if (a.remove_dc) K::remove_dc(v, red, tid, lf);
        K::fft(v, buf, tw, t);
        K::partners_prepare(v, buf, t);
        const int src = K::partner_lane(tid, t);
        float2 pz[T > 32 ? R : 1];
        if constexpr (T > 32) {
            static_for<0, R>([&](auto uc) {
                constexpr int u = decltype(uc)::value;
                pz[u] = K::template partner_at<u>(v, buf, t, src);
            });
        }
        __syncthreads();  // exchange buffers become output rows

        // ---------------- untangle into padded output rows
        // power: bins k < M/2 give X[k], X[N-k], X[M+k], X[M-k] (k = M/2 by
        // thread 0); half-complex: X[k] and X[k + M] for every slot
        float* orow = s_x + lf * OS;
        static_for<0, OUTK == OUT_HALF ? R : R / 2 + 1>([&](auto uc) {
            constexpr int u = decltype(uc)::value;
            float2 pu;
            if constexpr (T > 32) pu = pz[u];
            else pu = K::template partner_at<u>(v, buf, t, src);
            if constexpr (OUTK != OUT_HALF && u == R / 2) {
                if (t != 0) return;
            }
            const int k = t + u * T;
            float2 e, wo;
            K::untangle(v[u], pu, tw_get(tw, k, k), e, wo);
            const float2 xa = cadd(e, wo), xb = csub(e, wo);
            if constexpr (OUTK == OUT_HALF) {
                float2* o2 = reinterpret_cast<float2*>(orow);
                o2[k] = xa;
                o2[k + M] = xb;
            } else {
                const float pa = power_of<OUTK>(xa);
                orow[k] = pa;
                if (k != 0) orow[N - k] = pa;
                if constexpr (u != R / 2) {
                    const float pb = power_of<OUTK>(xb);
                    orow[M + k] = pb;
                    if (k != 0) orow[M - k] = pb;
                }
            }
        });
        __syncthreads();

        // ---------------- coalesced copy of the tile to HBM
        const uint64_t nf = (a.frames - fbase) < (uint64_t)FPC ? (a.frames - fbase) : (uint64_t)FPC;
        if constexpr (OUTK == OUT_HALF) {
            if (!a.dense) {
                // flat complex index < ohalf; rows of N complex = 2N floats
                float4* dst = reinterpret_cast<float4*>(a.out + 2 * fbase * (uint64_t)N);
                constexpr int cpr = N / 2;  // float4 per row
                const uint64_t lim4 = (2 * a.ohalf - 2 * fbase * (uint64_t)N) / 4;
                for (int q = tid; q < (int)nf * cpr; q += NT) {
                    const int jj = q / cpr, col = q - jj * cpr;
                    if ((uint64_t)q < lim4)
                        __stcs(dst + q, *reinterpret_cast<const float4*>(s_x + jj * OS + col * 4));
                }
            } else {
                float* dst = a.out + 2 * fbase * (uint64_t)(M + 1);
                constexpr int rw = 2 * (M + 1);
                for (int q = tid; q < (int)nf * rw; q += NT) {
                    const int jj = q / rw, col = q - jj * rw;
                    __stcs(dst + q, s_x[jj * OS + col]);
                }
            }
        } else {
            if (!a.dense) {
                float4* dst = reinterpret_cast<float4*>(a.out + fbase * (uint64_t)N);
                for (int q = tid; q < (int)nf * rows_chunks16; q += NT) {
                    const int jj = q / rows_chunks16, col = q - jj * rows_chunks16;
                    __stcs(dst + q, *reinterpret_cast<const float4*>(s_x + jj * OS + col * 4));
                }
            } else {
                float* dst = a.out + fbase * (uint64_t)(M + 1);
                constexpr int rw = M + 1;
                for (int q = tid; q < (int)nf * rw; q += NT) {
                    const int jj = q / rw, col = q - jj * rw;
                    __stcs(dst + q, s_x[jj * OS + col]);
                }
            }
        }
        (void)active;
        __syncthreads();  // output rows are exchange buffers again
    }
    cp_async_wait_all();
}

template <int EXP, int OUTK, bool STAGED>
cudaError_t launch_fused_t(const FusedArgs& a, int grid, cudaStream_t st)
{
    constexpr int threads = fused_cta_threads(EXP);
    if constexpr (STAGED) {
        if constexpr (fused_staged(EXP) && OUTK != OUT_PLANES) {
            constexpr size_t sm = staged_smem_bytes_ct(EXP, OUTK);
            auto k = stft_staged_kernel<EXP, OUTK>;
            const cudaError_t e = ensure_smem_attr<stft_staged_kernel<EXP, OUTK>>(sm);
            if (e != cudaSuccess) return e;
            k<<<grid, threads, sm, st>>>(a);
            return cudaGetLastError();
        } else {
            return cudaErrorInvalidValue;
        }
    } else {
        constexpr size_t sm = fused_smem_bytes_ct(EXP);
        auto k = stft_fused_kernel<EXP, OUTK>;
        const cudaError_t e = ensure_smem_attr<stft_fused_kernel<EXP, OUTK>>(sm);
        if (e != cudaSuccess) return e;
        k<<<grid, threads, sm, st>>>(a);
        return cudaGetLastError();
    }
}

template <int EXP, int OUTK, bool STAGED>
int occupancy_t()
{
    int blocks = 0;
    if constexpr (STAGED) {
        if constexpr (fused_staged(EXP) && OUTK != OUT_PLANES) {
            auto k = stft_staged_kernel<EXP, OUTK>;
            constexpr size_t sm = staged_smem_bytes_ct(EXP, OUTK);
            if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
                return 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k, fused_cta_threads(EXP), sm) != cudaSuccess)
                return 0;
        }
    } else {
        auto k = stft_fused_kernel<EXP, OUTK>;
        constexpr size_t sm = fused_smem_bytes_ct(EXP);
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k, fused_cta_threads(EXP), sm) != cudaSuccess)
            return 0;
    }
    return blocks;
}

// Dispatch over the output kind and I/O scheme for one exponent.
template <int EXP>
cudaError_t launch_fused_exp(int outk, bool staged, const FusedArgs& a, int grid, cudaStream_t st)
{
    if (staged) {
        switch (outk) {
        case OUT_POWER: return launch_fused_t<EXP, OUT_POWER, true>(a, grid, st);
        case OUT_POWER_SERIAL: return launch_fused_t<EXP, OUT_POWER_SERIAL, true>(a, grid, st);
        case OUT_HALF: return launch_fused_t<EXP, OUT_HALF, true>(a, grid, st);
        default: return cudaErrorInvalidValue;
        }
    }
    switch (outk) {
    case OUT_POWER: return launch_fused_t<EXP, OUT_POWER, false>(a, grid, st);
    case OUT_POWER_SERIAL: return launch_fused_t<EXP, OUT_POWER_SERIAL, false>(a, grid, st);
    case OUT_HALF: return launch_fused_t<EXP, OUT_HALF, false>(a, grid, st);
    case OUT_PLANES: return launch_fused_t<EXP, OUT_PLANES, false>(a, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int EXP>
int occupancy_exp(int outk, bool staged)
{
    if (staged) {
        switch (outk) {
        case OUT_POWER: return occupancy_t<EXP, OUT_POWER, true>();
        case OUT_POWER_SERIAL: return occupancy_t<EXP, OUT_POWER_SERIAL, true>();
        case OUT_HALF: return occupancy_t<EXP, OUT_HALF, true>();
        default: return 0;
        }
    }
    switch (outk) {
    case OUT_POWER: return occupancy_t<EXP, OUT_POWER, false>();
    case OUT_POWER_SERIAL: return occupancy_t<EXP, OUT_POWER_SERIAL, false>();
    case OUT_HALF: return occupancy_t<EXP, OUT_HALF, false>();
    case OUT_PLANES: return occupancy_t<EXP, OUT_PLANES, false>();
    default: return 0;
    }
}

}  // namespace ocs
