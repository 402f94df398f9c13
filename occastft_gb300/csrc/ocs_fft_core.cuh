// Device building blocks for the fused STFT kernels (sm_103a).
//
// The FFT of one frame of N real samples is done as an M = N/2 point complex
// FFT of z[m] = y[2m] + i*y[2m+1] followed by the real-input "untangle" step.
// The complex FFT is a Stockham autosort FFT: every thread of a frame group
// owns R complex values, stages have radix r_s | R, the first stage reads the
// frame straight from HBM and the last stage leaves X[t + u*T] in slot u of
// thread t, so no shared-memory pass is needed on either end.
//
// The math it replaces is the radix-2 Stockham of OKL/EXPCommon.okl:194-245 and
// OKL/EXP6.okl..EXP11.okl (one butterfly per thread per stage, cos/sin per
// butterfly); the result is the same DFT, X[k] = sum_n y[n] e^{-2 pi i k n / N}.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ocs {

// ------------------------------------------------------------------ plans
// Fused single-pass plan for window 2^exp: R values per thread, stage radices.
struct FusedCfg {
    int exp;
    int R;          // complex values per thread
    int nstages;
    int radix[6];
};

// Values per thread by window exponent (index 6..15); 32 values per thread
// give one shared-memory exchange up to 2^11 at the cost of registers.  The
// table is the measured choice; -DOCS_R_TABLE={...} builds a variant library
// for sweeps of the plan (loaded through OCS_LIBRARY).
#ifndef OCS_R_TABLE
#define OCS_R_TABLE {16, 8, 16, 16, 16, 32, 16, 16, 16, 32}
#endif
__host__ __device__ constexpr int fused_R(int exp)
{
    constexpr int tab[10] = OCS_R_TABLE;
    return (exp >= 6 && exp <= 15) ? tab[exp - 6] : 16;
}

__host__ __device__ constexpr FusedCfg fused_cfg(int exp)
{
    // M = 2^(exp-1) complex points; stages of radix R (<= 32) plus one remainder stage
    FusedCfg c{exp, fused_R(exp) < (1 << (exp - 1)) ? fused_R(exp) : (1 << (exp - 1)), 0, {1, 1, 1, 1, 1, 1}};
    const int lr = c.R == 32 ? 5 : (c.R == 16 ? 4 : (c.R == 8 ? 3 : (c.R == 4 ? 2 : 1)));
    int left = exp - 1;  // log2 M
    int s = 0;
    while (left >= lr) { c.radix[s++] = 1 << lr; left -= lr; }
    if (left > 0) c.radix[s++] = 1 << left;
    c.nstages = s;
    return c;
}

__host__ __device__ constexpr int fused_M(int exp) { return 1 << (exp - 1); }
__host__ __device__ constexpr int fused_T(int exp) { return fused_M(exp) / fused_cfg(exp).R; }
// Ns of stage s: product of the radices before it
__host__ __device__ constexpr int fused_Ns(int exp, int s)
{
    int ns = 1;
    for (int i = 0; i < s; ++i) ns *= fused_cfg(exp).radix[i];
    return ns;
}
// Twiddle table layout (float2 entries):
//   [0, M)                          W_N^k, the untangle twiddles
//   then for each stage s >= 1:     (r_s - 1) * Ns(s) entries, entry (m-1)*Ns + j = W_{Ns r}^{j m}
__host__ __device__ constexpr int fused_tw_offset(int exp, int s)
{
    int off = fused_M(exp);
    for (int i = 1; i < s; ++i) off += (fused_cfg(exp).radix[i] - 1) * fused_Ns(exp, i);
    return off;
}
__host__ __device__ constexpr int fused_tw_size(int exp) { return fused_tw_offset(exp, fused_cfg(exp).nstages); }

// threads per CTA and frames per CTA
__host__ __device__ constexpr int fused_cta_threads(int exp) { return fused_T(exp) >= 256 ? fused_T(exp) : 256; }
__host__ __device__ constexpr int fused_fpc(int exp) { return fused_cta_threads(exp) / fused_T(exp); }
// shared-memory exchange buffer per frame, in float2, padded one slot per 16
__host__ __device__ constexpr int fused_buf_stride(int exp) { return fused_M(exp) + fused_M(exp) / fused_cfg(exp).R + 1; }

// ------------------------------------------------------------------ math
// compile-time cos/sin of 2*pi*j/L by Taylor series (for in-register DFT constants)
__host__ __device__ constexpr double cx_sin(double x)
{
    double term = x, sum = x;
    for (int i = 1; i < 40; ++i) {
        term *= -x * x / ((2.0 * i) * (2.0 * i + 1.0));
        sum += term;
    }
    return sum;
}
__host__ __device__ constexpr double cx_cos(double x)
{
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 40; ++i) {
        term *= -x * x / ((2.0 * i - 1.0) * (2.0 * i));
        sum += term;
    }
    return sum;
}
constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr float kRsqrt2 = 0.70710678118654752440f;

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// a * W_L^J with W_L = exp(-2 pi i / L), J and L compile-time
template <int J, int L>
__device__ __forceinline__ float2 twc(float2 a)
{
    constexpr int j = ((J % L) + L) % L;
    if constexpr (j == 0) {
        return a;
    } else if constexpr (2 * j == L) {
        return make_float2(-a.x, -a.y);
    } else if constexpr (4 * j == L) {  // -i
        return make_float2(a.y, -a.x);
    } else if constexpr (4 * j == 3 * L) {  // +i
        return make_float2(-a.y, a.x);
    } else if constexpr (8 * j == L) {  // (1-i)/sqrt2
        return make_float2((a.x + a.y) * kRsqrt2, (a.y - a.x) * kRsqrt2);
    } else if constexpr (8 * j == 3 * L) {  // (-1-i)/sqrt2
        return make_float2((a.y - a.x) * kRsqrt2, -(a.x + a.y) * kRsqrt2);
    } else {
        constexpr float c = (float)cx_cos(kTwoPi * j / L);
        constexpr float s = (float)cx_sin(kTwoPi * j / L);
        // (x + iy)(c - is)
        return make_float2(a.x * c + a.y * s, a.y * c - a.x * s);
    }
}

constexpr int ilog2(int v) { return v <= 1 ? 0 : 1 + ilog2(v >> 1); }
constexpr int bitrev(int v, int bits)
{
    int r = 0;
    for (int i = 0; i < bits; ++i) r |= ((v >> i) & 1) << (bits - 1 - i);
    return r;
}

// One radix-2 DIF level over a register array view: blocks of size L at
// indices OFF + STRIDE * (b*L + j).  Recursion over L keeps every index a
// compile-time constant.
template <int R, int P, int OFF, int STRIDE, int L, int J>
struct DifLevel {
    static __device__ __forceinline__ void run_j(float2 (&v)[R], int /*unused*/)
    {
        if constexpr (J < L / 2) {
            // every block of this level
            DifLevel<R, P, OFF, STRIDE, L, J>::template run_blocks<0>(v);
            DifLevel<R, P, OFF, STRIDE, L, J + 1>::run_j(v, 0);
        }
    }
    template <int B>
    static __device__ __forceinline__ void run_blocks(float2 (&v)[R])
    {
        if constexpr (B < P / L) {
            constexpr int i0 = OFF + STRIDE * (B * L + J);
            constexpr int i1 = OFF + STRIDE * (B * L + J + L / 2);
            const float2 a = v[i0];
            const float2 b = v[i1];
            v[i0] = cadd(a, b);
            v[i1] = twc<J, L>(csub(a, b));
            run_blocks<B + 1>(v);
        }
    }
};

template <int R, int P, int OFF, int STRIDE, int L>
__device__ __forceinline__ void dif_levels(float2 (&v)[R])
{
    if constexpr (L >= 2) {
        DifLevel<R, P, OFF, STRIDE, L, 0>::run_j(v, 0);
        dif_levels<R, P, OFF, STRIDE, L / 2>(v);
    }
}

template <int R, int P, int OFF, int STRIDE, int K>
__device__ __forceinline__ void bitrev_gather(float2 (&v)[R], float2 (&tmp)[P])
{
    if constexpr (K < P) {
        tmp[K] = v[OFF + STRIDE * bitrev(K, ilog2(P))];
        bitrev_gather<R, P, OFF, STRIDE, K + 1>(v, tmp);
    }
}
template <int R, int P, int OFF, int STRIDE, int K>
__device__ __forceinline__ void scatter_back(float2 (&v)[R], const float2 (&tmp)[P])
{
    if constexpr (K < P) {
        v[OFF + STRIDE * K] = tmp[K];
        scatter_back<R, P, OFF, STRIDE, K + 1>(v, tmp);
    }
}

// In-place P-point DFT (natural order in and out) of v[OFF + STRIDE*m], m < P.
template <int R, int P, int OFF, int STRIDE>
__device__ __forceinline__ void dft_inreg(float2 (&v)[R])
{
    if constexpr (P > 1) {
        dif_levels<R, P, OFF, STRIDE, P>(v);
        float2 tmp[P];
        bitrev_gather<R, P, OFF, STRIDE, 0>(v, tmp);
        scatter_back<R, P, OFF, STRIDE, 0>(v, tmp);
    }
}

}  // namespace ocs
