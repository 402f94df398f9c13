// Packed FP32x2 building blocks (sm_100 and later): add/sub/mul/fma on a pair
// of FP32 lanes as one instruction, and complex DFTs run on two complex points
// per register pair.  Used where the FP32 kernels are bound by instruction
// issue (the paired-frame kernel at 2^10).
#pragma once
#include "stft_fused_kernel.cuh"

namespace ocs {
namespace x2 {

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 bc(float v) { return make_float2(v, v); }

// Two complex points: lane 0 is (re.x, im.x), lane 1 is (re.y, im.y).
struct C2 {
    float2 re, im;
};
__device__ __forceinline__ float2 lane0(const C2& v) { return make_float2(v.re.x, v.im.x); }
__device__ __forceinline__ float2 lane1(const C2& v) { return make_float2(v.re.y, v.im.y); }
__device__ __forceinline__ C2 pack(float2 l0, float2 l1) { return C2{make_float2(l0.x, l1.x), make_float2(l0.y, l1.y)}; }

// (a - b) * W_L^J in both lanes, W_L = exp(-2 pi i / L)
template <int J, int L>
__device__ __forceinline__ C2 diff_tw(const C2& a, const C2& b)
{
    constexpr int j = ((J % L) + L) % L;
    if constexpr (j == 0) {
        return C2{sub2(a.re, b.re), sub2(a.im, b.im)};
    } else if constexpr (2 * j == L) {
        return C2{sub2(b.re, a.re), sub2(b.im, a.im)};
    } else if constexpr (4 * j == L) {  // times -i
        return C2{sub2(a.im, b.im), sub2(b.re, a.re)};
    } else if constexpr (4 * j == 3 * L) {  // times +i
        return C2{sub2(b.im, a.im), sub2(a.re, b.re)};
    } else {
        const C2 d{sub2(a.re, b.re), sub2(a.im, b.im)};
        if constexpr (8 * j == L) {  // (1 - i) / sqrt 2
            return C2{mul2(add2(d.re, d.im), bc(kRsqrt2)), mul2(sub2(d.im, d.re), bc(kRsqrt2))};
        } else if constexpr (8 * j == 3 * L) {  // (-1 - i) / sqrt 2
            return C2{mul2(sub2(d.im, d.re), bc(kRsqrt2)), mul2(add2(d.re, d.im), bc(-kRsqrt2))};
        } else {
            constexpr float c = (float)cx_cos(kTwoPi * j / L);
            constexpr float s = (float)cx_sin(kTwoPi * j / L);
            // d (c - i s) = (re c + im s, im c - re s)
            return C2{fma2(d.im, bc(s), mul2(d.re, bc(c))), fma2(d.re, bc(-s), mul2(d.im, bc(c)))};
        }
    }
}

// P-point DFT of each lane, natural order in and out: radix-2 decimation in
// frequency, then the bit-reversal permutation as register renaming.
template <int P>
__device__ __forceinline__ void dft_lanes(C2 (&v)[P])
{
    static_for<0, ilog2(P)>([&](auto lc) {
        constexpr int L = P >> decltype(lc)::value;
        static_for<0, P / L>([&](auto bcn) {
            constexpr int b = decltype(bcn)::value;
            static_for<0, L / 2>([&](auto jc) {
                constexpr int j = decltype(jc)::value;
                constexpr int i0 = b * L + j, i1 = i0 + L / 2;
                const C2 x = v[i0], y = v[i1];
                v[i0] = C2{add2(x.re, y.re), add2(x.im, y.im)};
                v[i1] = diff_tw<j, L>(x, y);
            });
        });
    });
    C2 tmp[P];
    static_for<0, P>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        tmp[k] = v[bitrev(k, ilog2(P))];
    });
    static_for<0, P>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        v[k] = tmp[k];
    });
}

}  // namespace x2

}  // namespace ocs
