// Fused single-pass STFT for windows 2^6 .. 2^15 on sm_103a.
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

__device__ __forceinline__ float mag(float2 a, int serial)
{
    if (serial) {
        // the Serial runner's toPower(out, Real, Real): sqrt(R*R + R*R), no fused multiply-add
        const float rr = __fmul_rn(a.x, a.x);
        return __fsqrt_rn(__fadd_rn(rr, rr));
    }
    return __fsqrt_rn(__fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)));
}

template <int EXP, bool VEC2>
__global__ void __launch_bounds__(fused_cta_threads(EXP), (fused_cta_threads(EXP) >= 512 ? 1 : 512 / fused_cta_threads(EXP)))
stft_fused_kernel(const FusedArgs a)
{
    constexpr FusedCfg C = fused_cfg(EXP);
    constexpr int N = 1 << EXP;
    constexpr int M = N / 2;
    constexpr int R = C.R;
    constexpr int T = M / R;
    constexpr int FPC = fused_fpc(EXP);
    constexpr int BS = fused_buf_stride(EXP);
    constexpr int NS = C.nstages;
    constexpr unsigned FULL = 0xffffffffu;

    extern __shared__ float2 smem[];
    const int tid = threadIdx.x;
    const int lf = tid / T;
    const int t = tid - lf * T;
    float2* buf = smem + lf * BS;
    float* red = reinterpret_cast<float*>(smem + FPC * BS);

    const float2* __restrict__ tw = a.tw;
    const float2* __restrict__ win2 = reinterpret_cast<const float2*>(a.win);

    for (uint64_t fbase = (uint64_t)blockIdx.x * FPC; fbase < a.frames; fbase += (uint64_t)gridDim.x * FPC) {
        const uint64_t f = fbase + lf;
        const bool active = f < a.frames;
        float2 v[R];

        // ---------------- framing + window (one HBM read of the frame)
        {
            const uint64_t s = f * a.hop;
            const float* xs = a.x + s;
            if (active && s + N <= a.n) {
#pragma unroll
                for (int u = 0; u < R; ++u) {
                    const int c = t + u * T;
                    if constexpr (VEC2) {
                        v[u] = reinterpret_cast<const float2*>(xs)[c];
                    } else {
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
            if (win2 != nullptr) {
#pragma unroll
                for (int u = 0; u < R; ++u) {
                    const float2 w = win2[t + u * T];
                    v[u].x *= w.x;
                    v[u].y *= w.y;
                }
            }
        }

        // ---------------- DC removal: subtract the windowed frame's mean
        if (a.remove_dc) {
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

        // ---------------- stage 0 (no twiddles)
        {
            constexpr int r = C.radix[0];
            static_for<0, R / r>([&](auto qc) {
                constexpr int q = decltype(qc)::value;
                dft_inreg<R, r, q, R / r>(v);
            });
        }

        // ---------------- stages 1 .. NS-1: exchange through shared memory
        static_for<1, NS>([&](auto sc) {
            constexpr int s = decltype(sc)::value;
            constexpr int rp = C.radix[s - 1];       // previous stage radix
            constexpr int nsp = fused_Ns(EXP, s - 1);
            constexpr int r = C.radix[s];
            constexpr int ns = fused_Ns(EXP, s);
            constexpr int toff = fused_tw_offset(EXP, s);
            group_sync<T>();
            // write the previous stage's outputs at their Stockham positions
            static_for<0, R / rp>([&](auto qc) {
                constexpr int q = decltype(qc)::value;
                const int g = t + q * T;
                const int base = (g / nsp) * nsp * rp + (g % nsp);
                static_for<0, rp>([&](auto mc) {
                    constexpr int m = decltype(mc)::value;
                    buf[pad16(base + m * nsp)] = v[q + m * (R / rp)];
                });
            });
            group_sync<T>();
#pragma unroll
            for (int u = 0; u < R; ++u) v[u] = buf[pad16(t + u * T)];
            // twiddle and radix-r DFT
            static_for<0, R / r>([&](auto qc) {
                constexpr int q = decltype(qc)::value;
                const int j = (t + q * T) % ns;
                static_for<1, r>([&](auto mc) {
                    constexpr int m = decltype(mc)::value;
                    v[q + m * (R / r)] = cmul(v[q + m * (R / r)], tw[toff + (m - 1) * ns + j]);
                });
                dft_inreg<R, r, q, R / r>(v);
            });
        });

        // ---------------- real-input untangle: needs Z[M-k] for every owned k
        float2 pz[R];
        if constexpr (T <= 32) {
            const int lane = tid & 31;
            const int src = (lane & ~(T - 1)) | ((T - t) & (T - 1));
#pragma unroll
            for (int u = 0; u < R; ++u) {
                float2 p;
                p.x = __shfl_sync(FULL, v[R - 1 - u].x, src);
                p.y = __shfl_sync(FULL, v[R - 1 - u].y, src);
                pz[u] = (t == 0) ? v[(R - u) % R] : p;
            }
        } else {
            group_sync<T>();
#pragma unroll
            for (int u = 0; u < R; ++u) buf[pad16(t + u * T)] = v[u];
            group_sync<T>();
#pragma unroll
            for (int u = 0; u < R; ++u) {
                const float2 p = buf[pad16((T - t) + (R - 1 - u) * T)];
                pz[u] = (t == 0) ? v[(R - u) % R] : p;
            }
        }

        if (!active) continue;

        // ---------------- untangle + fused output store
        const int mode = a.mode;
        const int serial = a.serial_power;
        const int dense = a.dense;
#pragma unroll
        for (int u = 0; u < R; ++u) {
            const int k = t + u * T;
            const float2 zk = v[u];
            const float2 zc = make_float2(pz[u].x, -pz[u].y);  // conj(Z[M-k])
            const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
            const float2 d = csub(zk, zc);
            const float2 o = make_float2(0.5f * d.y, -0.5f * d.x);  // d / (2i)
            const float2 wo = cmul(tw[k], o);
            const float2 xa = cadd(e, wo);   // X[k]
            const float2 xb = csub(e, wo);   // X[k + M]
            if (mode == OCS_MODE_POWER) {
                if (!dense) {
                    float* row = a.out + f * (uint64_t)N;
                    __stcs(row + k, mag(xa, serial));
                    __stcs(row + k + M, mag(xb, serial));
                } else {
                    float* row = a.out + f * (uint64_t)(M + 1);
                    __stcs(row + k, mag(xa, serial));
                    if (k == 0) __stcs(row + M, mag(xb, serial));
                }
            } else if (mode == OCS_MODE_HALF_COMPLEX) {
                float2* o2 = reinterpret_cast<float2*>(a.out);
                if (!dense) {
                    const uint64_t flat = f * (uint64_t)N + k;
                    if (flat < a.ohalf) __stcs(o2 + flat, xa);
                    if (flat + M < a.ohalf) __stcs(o2 + flat + M, xb);
                } else {
                    float2* row = o2 + f * (uint64_t)(M + 1);
                    __stcs(row + k, xa);
                    if (k == 0) __stcs(row + M, xb);
                }
            } else {  // planes
                const uint64_t b = f * (uint64_t)N + k;
                a.out[b] = xa.x;
                a.out_im[b] = xa.y;
                a.out[b + M] = xb.x;
                a.out_im[b + M] = xb.y;
            }
        }
    }
}

// --------------------------------------------------------------- twiddles
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

template <int EXP, bool VEC2>
static cudaError_t launch_one(const FusedArgs& a, int grid, cudaStream_t st)
{
    constexpr int threads = fused_cta_threads(EXP);
    const size_t sm = fused_smem_bytes(EXP);
    auto k = stft_fused_kernel<EXP, VEC2>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k<<<grid, threads, sm, st>>>(a);
    return cudaGetLastError();
}

template <int EXP, bool VEC2>
static int occupancy_one()
{
    int blocks = 0;
    auto k = stft_fused_kernel<EXP, VEC2>;
    const size_t sm = fused_smem_bytes(EXP);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k, fused_cta_threads(EXP), sm) != cudaSuccess)
        return 0;
    return blocks;
}

size_t fused_smem_bytes(int exp)
{
    return (size_t)fused_fpc(exp) * fused_buf_stride(exp) * sizeof(float2) +
           (size_t)(fused_cta_threads(exp) / 32) * sizeof(float) + 16;
}

#define OCS_EXP_CASES(X) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15)

cudaError_t launch_fused(int exp, bool vec2, const FusedArgs& a, int grid, cudaStream_t st)
{
    switch (exp) {
#define X(E)                                                                      \
    case E:                                                                       \
        return vec2 ? launch_one<E, true>(a, grid, st) : launch_one<E, false>(a, grid, st);
        OCS_EXP_CASES(X)
#undef X
    default:
        return cudaErrorInvalidValue;
    }
}

int fused_occupancy(int exp, bool vec2)
{
    switch (exp) {
#define X(E) \
    case E:  \
        return vec2 ? occupancy_one<E, true>() : occupancy_one<E, false>();
        OCS_EXP_CASES(X)
#undef X
    default:
        return 0;
    }
}

int fused_frames_per_cta(int exp) { return fused_fpc(exp); }
int fused_twiddle_count(int exp) { return fused_tw_size(exp); }

cudaError_t build_twiddles(float2* tw, int exp, cudaStream_t st)
{
    const int n = fused_tw_size(exp);
    build_twiddles_kernel<<<(n + 255) / 256, 256, 0, st>>>(tw, exp);
    return cudaGetLastError();
}

}  // namespace ocs
