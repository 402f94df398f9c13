// Paired-frame fused STFT kernel (windows 2^6 .. 2^14, sm_103a).
//
// Two consecutive real frames a = 2p and b = 2p+1 ride in one N-point complex
// FFT, z[c] = y_a[c] + i y_b[c] (the classic "two real FFTs for one" identity):
//   A[k] = (Z[k] + conj Z[N-k]) / 2,   B[k] = (Z[k] - conj Z[N-k]) / (2i).
// Compared with one N/2-point FFT per frame plus the real-input untangle this
// needs no untangle twiddles, reads each window coefficient once for two
// frames, and with 32 values per thread needs a single shared-memory exchange
// up to N = 1024.  The 1/2 factors are folded into the window table (the
// table is pre-scaled by 1/2, an exact operation).
//
// Per frame it implements the same pipeline as the reference's
// Overlap_Common -> Window_* -> DCRemove_Common -> Stockham FFT -> toPower /
// toHalfComplexFormat (OKL/EXPCommon.okl:7-245, OKL/kernel.okl:178-218).
#pragma once
#include "stft_fused_kernel.cuh"

namespace ocs {

// ------------------------------------------------------------ plan
// A paired plan is named by an id: the window exponent, plus kPairR16 for the
// variant with 16 values per thread.  The one-request kernel at 2^12 runs that
// variant (a 16 . 16 . 16 plan at three CTAs per SM, 80 registers: power 305
// -> 316, half-complex 451 -> 485 Gsamples/s against 32 . 32 . 4); the batch
// keeps 32 values per thread there (its kernel stays at two CTAs per SM, and
// its 2^12 tiles measured 2.18 -> 2.25 ms with 16).  Every function below
// takes a plan id.  -DOCS_PAIR_R16_MASK=(1<<e | ...) and -DOCS_PAIR_MINB_R16
// build variant libraries with 16 values per thread at other windows.
#ifndef OCS_PAIR_R16_MASK
#define OCS_PAIR_R16_MASK 0
#endif
constexpr int kPairR16 = 32;
__host__ __device__ constexpr int pair_e(int pid) { return pid & 31; }  // window exponent
__host__ __device__ constexpr bool pair_r16(int pid)
{
    return (pid & kPairR16) != 0 || (((OCS_PAIR_R16_MASK) >> (pid & 31)) & 1);
}
__host__ __device__ constexpr int pair_R(int pid) { return pair_e(pid) <= 6 || pair_r16(pid) ? 16 : 32; }
__host__ __device__ constexpr int pair_min_blocks(int pid);

__host__ __device__ constexpr FusedCfg pair_cfg(int pid)
{
    FusedCfg c{pair_e(pid), pair_R(pid), 0, {1, 1, 1, 1, 1, 1}};
    const int lr = c.R == 32 ? 5 : 4;
    int left = pair_e(pid);  // log2 of the complex FFT size N
    int s = 0;
    while (left >= lr) { c.radix[s++] = 1 << lr; left -= lr; }
    if (left > 0) c.radix[s++] = 1 << left;
    c.nstages = s;
    return c;
}
__host__ __device__ constexpr int pair_T(int pid) { return (1 << pair_e(pid)) / pair_R(pid); }
__host__ __device__ constexpr int pair_Ns(int pid, int s)
{
    int ns = 1;
    for (int i = 0; i < s; ++i) ns *= pair_cfg(pid).radix[i];
    return ns;
}
// twiddle table: for each stage s >= 1, (r_s - 1) * Ns(s) entries, (m-1)*Ns + j = W_{Ns r}^{j m}
__host__ __device__ constexpr int pair_tw_offset(int pid, int s)
{
    int off = 0;
    for (int i = 1; i < s; ++i) off += (pair_cfg(pid).radix[i] - 1) * pair_Ns(pid, i);
    return off;
}
__host__ __device__ constexpr int pair_tw_size(int pid)
{
    return pair_tw_offset(pid, pair_cfg(pid).nstages) > 0 ? pair_tw_offset(pid, pair_cfg(pid).nstages) : 1;
}
__host__ __device__ constexpr int pair_cta_threads(int pid) { return pair_T(pid) >= 256 ? pair_T(pid) : 256; }
__host__ __device__ constexpr int pair_ppc(int pid) { return pair_cta_threads(pid) / pair_T(pid); }  // pairs per CTA
__host__ __device__ constexpr int pair_buf_stride(int pid)
{
    return (1 << pair_e(pid)) + (1 << pair_e(pid)) / pair_R(pid) + 1;
}
__host__ __device__ constexpr bool pair_tables_in_smem(int pid) { return pair_e(pid) <= 11; }
__host__ __device__ constexpr bool pair_supported(int pid) { return pair_e(pid) >= 6 && pair_e(pid) <= 14; }
// 2 x 256 threads per SM below 2^14 (R = 16 at 2^10, three 256-thread CTAs
// of up to 80 registers, measured 300 against 390 Gsamples/s: the extra
// block-wide exchange costs more than the occupancy gains); the 16-value
// plans of 2^12 and up have as many exchanges as the 32-value ones and run
// three CTAs per SM
__host__ __device__ constexpr int pair_min_blocks(int pid)
{
#ifdef OCS_PAIR_MINB_R16
    if (((OCS_PAIR_R16_MASK) >> pair_e(pid)) & 1) return OCS_PAIR_MINB_R16;
#endif
    if ((pid & kPairR16) != 0) return 3;
    return pair_cta_threads(pid) >= 512 ? 1 : 512 / pair_cta_threads(pid);
}
// Twiddle entries copied to shared memory: the whole table up to 2^11; above,
// the first exchange stage's (31 x 32 entries, 7.9 KB), which next to the
// window still fits beside the exchange buffers at the same occupancy; the
// later stages' twiddles are read through L1.
__host__ __device__ constexpr int pair_smem_tw_entries(int pid)
{
    return pair_tables_in_smem(pid) ? pair_tw_size(pid)
                                    : (pair_cfg(pid).nstages > 2 ? pair_tw_offset(pid, 2) : pair_tw_size(pid));
}
// The window joins them except at 2^13, where its 32 KB would take from L1
// what the overlapping frames' loads reuse (2^13 power: 278 Gsamples/s with
// the window read through L1, 254 with it in shared memory).
__host__ __device__ constexpr bool pair_smem_window(int pid) { return pair_e(pid) != 13; }
// From 2^12 the later stages' twiddles come from a two-level table in shared
// memory, W_N^e = lo[e & 127] * hi[e >> 7] (128 + N/128 entries), chained
// between sparse lookups as in the one-frame kernels, instead of the plan
// table through L1 (at 2^14 that table is 123 KB and misses L1): 2^12 276 ->
// 280, 2^13 268 -> 278, 2^14 211 -> 218 Gsamples/s (power).
__host__ __device__ constexpr bool pair_tw2l(int pid) { return pair_e(pid) >= 12; }
__host__ __device__ constexpr size_t pair_tw2l_bytes(int pid)
{
    return pair_tw2l(pid) ? (128 + (1 << pair_e(pid)) / 128) * 8 : 0;
}
__host__ __device__ constexpr size_t pair_tab_bytes(int pid)
{
    return (size_t)pair_smem_tw_entries(pid) * 8 + pair_tw2l_bytes(pid) +
           (pair_smem_window(pid) ? (size_t)(1 << pair_e(pid)) * 4 : 0);
}
__host__ __device__ constexpr size_t pair_smem_bytes_ct(int pid)
{
    return (size_t)pair_ppc(pid) * pair_buf_stride(pid) * 8 + pair_tab_bytes(pid) +
           (size_t)(pair_cta_threads(pid) / 32) * 8 + 16;
}

template <int EXP>  // a plan id
struct PairCore {
    static constexpr FusedCfg C = pair_cfg(EXP);
    static constexpr int N = 1 << pair_e(EXP);
    static constexpr int R = C.R;
    static constexpr int T = N / R;
    static constexpr int NS = C.nstages;
    static constexpr int LP = ilog2(R);
    static constexpr unsigned FULL = 0xffffffffu;
    static __device__ __forceinline__ int pd(int i) { return padl<LP>(i); }

    // subtract each frame's mean: frame a is the real part, frame b the imaginary part
    static __device__ __forceinline__ void remove_dc(float2 (&v)[R], float2* red, int tid, int lp)
    {
        float sa = 0.0f, sb = 0.0f;
#pragma unroll
        for (int u = 0; u < R; ++u) {
            sa += v[u].x;
            sb += v[u].y;
        }
        if constexpr (T <= 32) {
#pragma unroll
            for (int o = T / 2; o > 0; o >>= 1) {
                sa += __shfl_xor_sync(FULL, sa, o);
                sb += __shfl_xor_sync(FULL, sb, o);
            }
        } else {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sa += __shfl_xor_sync(FULL, sa, o);
                sb += __shfl_xor_sync(FULL, sb, o);
            }
            constexpr int WPF = T / 32;
            if ((tid & 31) == 0) red[tid >> 5] = make_float2(sa, sb);
            __syncthreads();
            sa = 0.0f;
            sb = 0.0f;
#pragma unroll
            for (int w = 0; w < WPF; ++w) {
                const float2 r = red[lp * WPF + w];
                sa += r.x;
                sb += r.y;
            }
            __syncthreads();
        }
        const float ma = sa * (1.0f / (float)N), mb = sb * (1.0f / (float)N);
#pragma unroll
        for (int u = 0; u < R; ++u) {
            v[u].x -= ma;
            v[u].y -= mb;
        }
    }

    // tws: shared-memory copy of the first pair_smem_tw_entries(EXP) twiddles;
    // twg: the whole table in global memory (same indexing); tw2: the
    // two-level table (pair_tw2l) that replaces twg
    static __device__ __forceinline__ void fft(float2 (&v)[R], float2* buf, const float2* tws, const float2* twg,
                                               const TwTwoLevel& tw2, int t)
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
            constexpr int rp = C.radix[s - 1];
            constexpr int nsp = pair_Ns(EXP, s - 1);
            constexpr int r = C.radix[s];
            constexpr int ns = pair_Ns(EXP, s);
            constexpr int toff = pair_tw_offset(EXP, s);
            const float2* const tw = pair_tw_offset(EXP, s + 1) <= pair_smem_tw_entries(EXP) ? tws : twg;
            group_sync<T>();
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
            constexpr bool in_smem = pair_tw_offset(EXP, s + 1) <= pair_smem_tw_entries(EXP);
            constexpr int ef = N / (ns * r);  // W_{ns r}^{j m} = W_N^{j m ef}
            static_for<0, R / r>([&](auto qc) {
                constexpr int q = decltype(qc)::value;
                const int j = (t + q * T) % ns;
                if constexpr (!in_smem && pair_tw2l(EXP)) {
                    // a two-level lookup every 8th m, products with W^{j ef} between
                    float2 b = make_float2(1.0f, 0.0f), w = b;
                    static_for<1, r>([&](auto mc) {
                        constexpr int m = decltype(mc)::value;
                        if constexpr ((m - 1) % 8 == 0) {
                            w = tw_get(tw2, 0, j * m * ef);
                            if constexpr (m == 1) b = w;
                        } else {
                            w = cmul(w, b);
                        }
                        v[q + m * (R / r)] = cmul(v[q + m * (R / r)], w);
                    });
                } else {
                    static_for<1, r>([&](auto mc) {
                        constexpr int m = decltype(mc)::value;
                        v[q + m * (R / r)] = cmul(v[q + m * (R / r)], tw[toff + (m - 1) * ns + j]);
                    });
                }
                dft_inreg<R, r, q, R / r>(v);
            });
        });
    }

    static __device__ __forceinline__ void partners_prepare(const float2 (&v)[R], float2* buf, int t)
    {
        if constexpr (T > 32) {
            group_sync<T>();
#pragma unroll
            for (int u = 0; u < R; ++u) buf[pd(t + u * T)] = v[u];
            group_sync<T>();
        }
    }
    // Z[N - (t + U*T)]
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
};

template <int EXP>
__device__ __forceinline__ void pair_tables(const FusedArgs& a, float2* s_tab, int tid, const float*& win,
                                            TwTwoLevel& tw2)
{
    constexpr int TWN = pair_smem_tw_entries(EXP);
    constexpr int N = 1 << pair_e(EXP);
    for (int i = tid; i < TWN; i += blockDim.x) s_tab[i] = a.tw[i];
    float2* s2 = s_tab + TWN;
    if constexpr (pair_tw2l(EXP)) {
        // lo[e] = W_N^e (e < 128), hi[h] = W_N^(128 h) (h < N / 128)
        for (int i = tid; i < 128 + N / 128; i += blockDim.x) {
            const int e = i < 128 ? i : (i - 128) * 128;
            double sn, cs;
            sincospi(2.0 * (double)e / (double)N, &sn, &cs);
            s2[i] = make_float2((float)cs, (float)(-sn));
        }
        tw2 = TwTwoLevel{s2, s2 + 128};
    }
    if constexpr (pair_smem_window(EXP)) {
        float* sw = reinterpret_cast<float*>(reinterpret_cast<char*>(s2) + pair_tw2l_bytes(EXP));
        for (int i = tid; i < N; i += blockDim.x) sw[i] = a.win[i];
        win = sw;
    } else {
        win = a.win;
    }
    __syncthreads();
}

template <int EXP, int OUTK>
__device__ __forceinline__ void pair_group(const FusedArgs& a, uint64_t pbase, float2* buf, float2* red,
                                           const float2* tws, const TwTwoLevel& tw2, const float* win, int tid,
                                           int lp, int t);

template <int EXP, int OUTK>
__global__ void __launch_bounds__(pair_cta_threads(EXP), pair_min_blocks(EXP))
stft_pair_kernel(const FusedArgs a)
{
    using K = PairCore<EXP>;
    constexpr int T = K::T;
    constexpr int PPC = pair_ppc(EXP);
    constexpr int BS = pair_buf_stride(EXP);

    extern __shared__ float2 smem[];
    const int tid = threadIdx.x;
    const int lp = tid / T;
    const int t = tid - lp * T;
    float2* buf = smem + lp * BS;
    float2* s_tab = smem + PPC * BS;
    float2* red = reinterpret_cast<float2*>(reinterpret_cast<char*>(s_tab) + pair_tab_bytes(EXP));
    const float* win;
    TwTwoLevel tw2{nullptr, nullptr};
    pair_tables<EXP>(a, s_tab, tid, win, tw2);

    const uint64_t pairs = (a.frames + 1) / 2;
    for (uint64_t pbase = (uint64_t)blockIdx.x * PPC; pbase < pairs; pbase += (uint64_t)gridDim.x * PPC) {
        // L2 prefetch of the pair this group takes next: samples of frames 2q and 2q + 1
        const uint64_t q = pbase + (uint64_t)gridDim.x * PPC + lp;
        if (t == 0 && q < pairs) {
            const uint64_t s0 = 2 * q * a.hop;
            const uint64_t end = s0 + a.hop + (uint64_t)(1 << pair_e(EXP));
            prefetch_l2_span(a.x, s0, end < a.n ? end : a.n);
        }
        pair_group<EXP, OUTK>(a, pbase, buf, red, s_tab, tw2, win, tid, lp, t);
    }
}

// One CTA iteration: pairs pbase .. pbase + PPC - 1 (frames 2p, 2p + 1 below
// a.frames); buf is this thread's pair buffer, tws the shared-memory twiddles.
template <int EXP, int OUTK>
__device__ __forceinline__ void pair_group(const FusedArgs& a, uint64_t pbase, float2* buf, float2* red,
                                           const float2* tws, const TwTwoLevel& tw2, const float* win, int tid,
                                           int lp, int t)
{
    using K = PairCore<EXP>;
    constexpr int N = K::N, R = K::R, T = K::T;
    constexpr int H = N / 2;
    {
        const uint64_t p = pbase + lp;
        const uint64_t fa = 2 * p, fb = 2 * p + 1;
        const bool act_a = fa < a.frames;
        const bool act_b = fb < a.frames;
        float2 v[R];

        // ---------------- framing + window of both frames
        {
            const uint64_t sa = fa * a.hop;
            const uint64_t sb = sa + a.hop;
            const float* xa = a.x + sa;
            const float* xb = a.x + sb;
            if (pair_e(EXP) <= 12 && act_b && sb + N <= a.n && a.hop == (uint64_t)(N / 2)) {
                // frame b starts N/2 = (R/2) T samples after frame a: its slots
                // u < R/2 are frame a's slots u + R/2, so only half of them load
                // (1e8 samples, power: 2^9 377 -> 386, 2^10 392 -> 393, 2^12
                // 286 -> 291 Gsamples/s; at 2^13 it measured 278 -> 264 and
                // at 2^14 no change, so those keep loading both frames)
#pragma unroll
                for (int u = 0; u < R; ++u) v[u].x = xa[t + u * T];
#pragma unroll
                for (int u = R / 2; u < R; ++u) v[u].y = xb[t + u * T];
#pragma unroll
                for (int u = 0; u < R / 2; ++u) v[u].y = v[u + R / 2].x;
            } else if (pair_e(EXP) <= 12 && act_b && sb + N <= a.n && a.hop == (uint64_t)(N / 4)) {
                // overlap 0.75: frame b's slots u < 3R/4 are frame a's slots u + R/4
#pragma unroll
                for (int u = 0; u < R; ++u) v[u].x = xa[t + u * T];
#pragma unroll
                for (int u = 3 * R / 4; u < R; ++u) v[u].y = xb[t + u * T];
#pragma unroll
                for (int u = 0; u < 3 * R / 4; ++u) v[u].y = v[u + R / 4].x;
            } else if (act_b && sb + N <= a.n) {
#pragma unroll
                for (int u = 0; u < R; ++u) {
                    const int c = t + u * T;
                    v[u] = make_float2(xa[c], xb[c]);
                }
            } else {
#pragma unroll
                for (int u = 0; u < R; ++u) {
                    const int c = t + u * T;
                    const float ra = (act_a && sa + c < a.n) ? xa[c] : 0.0f;
                    const float rb = (act_b && sb + c < a.n) ? xb[c] : 0.0f;
                    v[u] = make_float2(ra, rb);
                }
            }
#pragma unroll
            for (int u = 0; u < R; ++u) {
                const float w = win[t + u * T];
                v[u].x *= w;
                v[u].y *= w;
            }
        }
        if (a.remove_dc) K::remove_dc(v, red, tid, lp);
        K::fft(v, buf, tws, a.tw, tw2, t);
        K::partners_prepare(v, buf, t);
        const int src = K::partner_lane(tid, t);

        // ---------------- separate the two spectra and store
        // slots u < R/2 carry k = t + u*T < N/2; thread 0 also owns k = N/2 (slot R/2)
        static_for<0, R / 2 + 1>([&](auto uc) {
            constexpr int u = decltype(uc)::value;
            const float2 pz = K::template partner_at<u>(v, buf, t, src);
            if (u == R / 2 && t != 0) return;
            const int k = t + u * T;
            const float2 z = v[u];
            const float2 A = make_float2(z.x + pz.x, z.y - pz.y);  // frame a, bin k
            const float2 B = make_float2(z.y + pz.y, pz.x - z.x);  // frame b, bin k
            if constexpr (OUTK == OUT_POWER || OUTK == OUT_POWER_SERIAL) {
                const float pa = power_of<OUTK>(A);
                const float pb = power_of<OUTK>(B);
                if (!a.dense) {
                    float* ra = a.out + fa * (uint64_t)N;
                    // slots 0 < u < R/2 hold T <= k < H: both mirror bins exist
                    constexpr bool inner = u != 0 && u != R / 2;
                    const bool mirror = inner || (k != 0 && k != H);
                    if (act_b) {  // both frames of the pair (act_b implies act_a)
                        __stcs(ra + k, pa);
                        __stcs(ra + N + k, pb);
                        if (mirror) {
                            __stcs(ra + (N - k), pa);
                            __stcs(ra + N + (N - k), pb);
                        }
                    } else if (act_a) {
                        __stcs(ra + k, pa);
                        if (mirror) __stcs(ra + (N - k), pa);
                    }
                } else {
                    float* ra = a.out + fa * (uint64_t)(H + 1);
                    if (act_a) __stcs(ra + k, pa);
                    if (act_b) __stcs(ra + (H + 1) + k, pb);
                }
            } else if constexpr (OUTK == OUT_HALF) {
                float2* o2 = reinterpret_cast<float2*>(a.out);
                if (!a.dense) {
                    const uint64_t fla = fa * (uint64_t)N;
                    const uint64_t flb = fla + N;
                    if (act_a && fla + k < a.ohalf) __stcs(o2 + fla + k, A);
                    if (act_a && k != 0 && k != H && fla + (N - k) < a.ohalf)
                        __stcs(o2 + fla + (N - k), make_float2(A.x, -A.y));
                    if (act_b && flb + k < a.ohalf) __stcs(o2 + flb + k, B);
                    if (act_b && k != 0 && k != H && flb + (N - k) < a.ohalf)
                        __stcs(o2 + flb + (N - k), make_float2(B.x, -B.y));
                } else {
                    float2* ra = o2 + fa * (uint64_t)(H + 1);
                    if (act_a) __stcs(ra + k, A);
                    if (act_b) __stcs(ra + (H + 1) + k, B);
                }
            }
        });
    }
}

template <int EXP, int OUTK>
cudaError_t launch_pair_t(const FusedArgs& a, int grid, cudaStream_t st)
{
    if constexpr (pair_supported(EXP) && OUTK != OUT_PLANES) {
        constexpr int threads = pair_cta_threads(EXP);
        constexpr size_t sm = pair_smem_bytes_ct(EXP);
        auto k = stft_pair_kernel<EXP, OUTK>;
        const cudaError_t e = ensure_smem_attr<stft_pair_kernel<EXP, OUTK>>(sm);
        if (e != cudaSuccess) return e;
        k<<<grid, threads, sm, st>>>(a);
        return cudaGetLastError();
    } else {
        return cudaErrorInvalidValue;
    }
}

template <int EXP, int OUTK>
int occupancy_pair_t()
{
    int blocks = 0;
    if constexpr (pair_supported(EXP) && OUTK != OUT_PLANES) {
        auto k = stft_pair_kernel<EXP, OUTK>;
        constexpr size_t sm = pair_smem_bytes_ct(EXP);
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k, pair_cta_threads(EXP), sm) != cudaSuccess)
            return 0;
    }
    return blocks;
}

template <int EXP>
cudaError_t launch_pair_exp(int outk, const FusedArgs& a, int grid, cudaStream_t st)
{
    switch (outk) {
    case OUT_POWER: return launch_pair_t<EXP, OUT_POWER>(a, grid, st);
    case OUT_POWER_SERIAL: return launch_pair_t<EXP, OUT_POWER_SERIAL>(a, grid, st);
    case OUT_HALF: return launch_pair_t<EXP, OUT_HALF>(a, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int EXP>
int occupancy_pair_exp(int outk)
{
    switch (outk) {
    case OUT_POWER: return occupancy_pair_t<EXP, OUT_POWER>();
    case OUT_POWER_SERIAL: return occupancy_pair_t<EXP, OUT_POWER_SERIAL>();
    case OUT_HALF: return occupancy_pair_t<EXP, OUT_HALF>();
    default: return 0;
    }
}

}  // namespace ocs
