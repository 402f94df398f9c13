// Tensor-core split-precision STFT (tcgen05, sm_103a), windows N = r*r with
// r = 16 or 32 (N = 256, 1024).
//
// Per frame the N-point DFT of the real windowed frame y is a four-step FFT:
//   pass 1  Y[g][k1] = sum_m y[g + r m] W_r^{m k1}          (r-point DFTs over m)
//   twiddle Y[g][k1] *= W_N^{g k1}
//   pass 2  X[k1 + r k2] = sum_g Y[g][k1] W_r^{g k2}         (r-point DFTs over g)
// Both passes are GEMMs on the 5th-generation tensor cores: the data is the A
// operand in shared memory, MN-major, which is exactly how the frame's samples
// (pass 1) and the pass-1 results (pass 2) come out of the threads, and the
// r-point DFT matrix (as a real 2r x r or 2r x 2r matrix) is the K-major B
// operand.  Accumulators (FP32) live in tensor memory and are read back with
// tcgen05.ld for the epilogues (twiddle + re-split; power / half-complex).
//
// Precision: every operand is split into fp16 hi + lo parts and each product
// is taken as hi*hi + hi*lo + lo*hi (FP32 accumulate).  Frames are scaled by a
// power of two so their peak sits near 2^14 (exact); pass-1 results are scaled
// by 1/r (exact) before the second split.
//
// Tile: 128 GEMM rows = 128/r frames.  One CTA of 128 threads (4 warps);
// thread i owns GEMM row i in both passes (TMEM lane i).  Waits on the MMA
// completion barrier are bounded; on a timeout the kernel records an error,
// frees its tensor memory and returns.
#include "ocs_kernels.h"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>
#include <mutex>

namespace ocs {
namespace {

constexpr uint32_t kSpinLimit = 1u << 28;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor: start, leading / stride byte
// offsets (16-byte units), descriptor version 1, 128-byte swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// instruction descriptor, kind::f16: fp16 A and B, fp32 D, A MN-major, B K-major
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N)
{
    return (1u << 4)                       // D format f32
           | (0u << 7) | (0u << 10)       // A, B format f16
           | (1u << 15)                    // A MN-major
           | (0u << 16)                    // B K-major
           | ((uint32_t)(N >> 3) << 17)   //
           | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity)
{
    const uint32_t a = smem_u32(mbar);
    for (uint32_t i = 0; i < kSpinLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float2 cmul2(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// fp16 hi/lo split of 8 floats into two 16-byte chunks
__device__ __forceinline__ void split8(const float (&x)[8], uint4& hi, uint4& lo)
{
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const __half a = __float2half_rn(x[2 * i]), b = __float2half_rn(x[2 * i + 1]);
        const __half c = __float2half_rn(x[2 * i] - __half2float(a));
        const __half d = __float2half_rn(x[2 * i + 1] - __half2float(b));
        h[i] = (uint32_t)__half_as_ushort(a) | ((uint32_t)__half_as_ushort(b) << 16);
        l[i] = (uint32_t)__half_as_ushort(c) | ((uint32_t)__half_as_ushort(d) << 16);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// Byte offset of element (mn, k) in an MN-major, 128-byte-swizzled operand of
// 128 MN-rows: atoms of 64 MN x 8 K (1024 B), MN atoms 1024 B apart, K atoms
// 2048 B apart.  The swizzle XORs the 16-byte chunk with the K row (mod 8).
__device__ __forceinline__ uint32_t mn_off(int mn, int k)
{
    const int chunk = (mn & 63) >> 3;
    return (uint32_t)((mn >> 6) * 1024 + (k >> 3) * 2048 + (k & 7) * 128 + ((chunk ^ (k & 7)) << 4) + ((mn & 7) << 1));
}

// Byte offset of element (n, k) in a K-major, 128-byte-swizzled operand with
// K <= 64: rows of 128 bytes, 8-row atoms 1024 B apart.
__device__ __forceinline__ uint32_t k_off(int n, int k)
{
    const int chunk = k >> 3;
    return (uint32_t)((n >> 3) * 1024 + (n & 7) * 128 + ((chunk ^ (n & 7)) << 4) + ((k & 7) << 1));
}

template <int R>
struct TcCfg {
    static constexpr int N = R * R;
    static constexpr int FPT = 128 / R;                 // frames per tile
    static constexpr int K1 = R;                        // pass-1 K: real inputs
    static constexpr int K2 = 2 * R;                    // pass-2 K: re and im inputs
    static constexpr int NO = 2 * R;                    // outputs per pass: re/im interleaved
    static constexpr uint32_t A1_BYTES = 2 * (K1 / 8) * 2048;  // hi + lo, 128 rows
    static constexpr uint32_t A2_BYTES = 2 * (K2 / 8) * 2048;
    static constexpr uint32_t B1_BYTES = 2 * NO * 128;  // hi + lo, K <= 64 -> one 128-B row each
    static constexpr uint32_t B2_BYTES = 2 * NO * 128;
    static constexpr uint32_t TW_BYTES = N * 8;
    static constexpr uint32_t OFF_A1 = 0;
    static constexpr uint32_t OFF_A2 = OFF_A1 + A1_BYTES;
    static constexpr uint32_t OFF_B1 = OFF_A2 + A2_BYTES;
    static constexpr uint32_t OFF_B2 = OFF_B1 + B1_BYTES;
    static constexpr uint32_t OFF_TW = OFF_B2 + B2_BYTES;
    static constexpr uint32_t OFF_MISC = OFF_TW + TW_BYTES;  // 2 mbarriers, tmem slot, frame scales
    static constexpr uint32_t SMEM = OFF_MISC + 256 + 1024;  // + slack to 1024-align the base
    static constexpr uint32_t TMEM_COLS = 2 * NO <= 32 ? 32 : (2 * NO <= 64 ? 64 : (2 * NO <= 128 ? 128 : 256));
    static_assert(K2 <= 64, "pass-2 K of one 128-byte row");
};

template <int R, int OUTK>
__global__ void __launch_bounds__(128, 1) stft_tc_kernel(const FusedArgs a, int* err)
{
    using C = TcCfg<R>;
    constexpr int N = C::N;
    constexpr int FPT = C::FPT;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* A1 = sm + C::OFF_A1;
    unsigned char* A2 = sm + C::OFF_A2;
    unsigned char* B1 = sm + C::OFF_B1;
    unsigned char* B2 = sm + C::OFF_B2;
    float2* TW = reinterpret_cast<float2*>(sm + C::OFF_TW);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + C::OFF_MISC);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + C::OFF_MISC + 16);
    float* fscale = reinterpret_cast<float*>(sm + C::OFF_MISC + 32);  // per-frame 1/scale, FPT entries
    int* abort_flag = reinterpret_cast<int*>(sm + C::OFF_MISC + 24);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // ---------------- set-up: barriers, tensor memory, DFT matrices, twiddles
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[1])));
        *abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(C::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    // B1: rows 2k1 (re), 2k1+1 (im) of the real-input r-point DFT, K = m
    for (int e = tid; e < C::NO * C::K1; e += 128) {
        const int row = e / C::K1, m = e % C::K1, k1 = row >> 1;
        double s, c;
        sincospi(2.0 * (double)((m * k1) % R) / (double)R, &s, &c);
        const float w = (row & 1) ? (float)(-s) : (float)c;
        const __half h = __float2half_rn(w), l = __float2half_rn(w - __half2float(h));
        *reinterpret_cast<__half*>(B1 + k_off(row, m)) = h;
        *reinterpret_cast<__half*>(B1 + C::B1_BYTES / 2 + k_off(row, m)) = l;
    }
    // B2: complex r-point DFT as a real matrix; K = g (re part, k < R) and g (im part, k >= R)
    for (int e = tid; e < C::NO * C::K2; e += 128) {
        const int row = e / C::K2, k = e % C::K2, k2 = row >> 1, g = k % R;
        double s, c;
        sincospi(2.0 * (double)((g * k2) % R) / (double)R, &s, &c);
        // (yr + i yi)(c - i s): re = yr c + yi s, im = yi c - yr s
        float w;
        if ((row & 1) == 0) w = (k < R) ? (float)c : (float)s;
        else w = (k < R) ? (float)(-s) : (float)c;
        const __half h = __float2half_rn(w), l = __float2half_rn(w - __half2float(h));
        *reinterpret_cast<__half*>(B2 + k_off(row, k)) = h;
        *reinterpret_cast<__half*>(B2 + C::B2_BYTES / 2 + k_off(row, k)) = l;
    }
    // twiddles W_N^{g k1}
    for (int e = tid; e < N; e += 128) {
        const int g = e / R, k1 = e % R;
        double s, c;
        sincospi(2.0 * (double)((g * k1) % N) / (double)N, &s, &c);
        TW[e] = make_float2((float)c, (float)(-s));
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t d1 = tmem, d2 = tmem + C::NO;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    constexpr uint32_t ID = idesc_f16(128, C::NO);
    const uint32_t a1 = smem_u32(A1), a2 = smem_u32(A2), b1 = smem_u32(B1), b2 = smem_u32(B2);

    const uint64_t ntiles = (a.frames + FPT - 1) / FPT;
    uint32_t phase = 0, phase1 = 0;  // parities of the pass-1 and pass-2 barriers
    bool aborted = false;
    for (uint64_t tile = blockIdx.x; tile < ntiles && !aborted; tile += gridDim.x) {
        const uint64_t f0 = tile * FPT;
        // ---------------- load + window + DC + scale + split -> A1 (one warp per frame)
        for (int lf = warp; lf < FPT; lf += 4) {
            const uint64_t f = f0 + lf;
            const bool act = f < a.frames;
            const uint64_t s0 = f * a.hop;
            float x[N / 32];
            float sum = 0.0f;
#pragma unroll
            for (int j = 0; j < N / 256; ++j) {  // lane owns samples [8c, 8c+8), c = lane + 32 j
                const int c = lane + 32 * j;
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int i = 8 * c + q;
                    const uint64_t gi = s0 + i;
                    float v = (act && gi < a.n) ? a.x[gi] : 0.0f;
                    if (a.win) v *= a.win[i];
                    x[8 * j + q] = v;
                    sum += v;
                }
            }
            if (a.remove_dc) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
                const float mean = sum * (1.0f / (float)N);
#pragma unroll
                for (int i = 0; i < N / 32; ++i) x[i] -= mean;
            }
            float mx = 0.0f;
#pragma unroll
            for (int i = 0; i < N / 32; ++i) mx = fmaxf(mx, fabsf(x[i]));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            int e2 = 0;
            if (mx > 0.0f) frexpf(mx, &e2);  // mx in [2^(e2-1), 2^e2)
            const float sc = ldexpf(1.0f, 14 - e2);
            if (lane == 0) fscale[lf] = ldexpf(1.0f, e2 - 14);
#pragma unroll
            for (int j = 0; j < N / 256; ++j) {
                const int c = lane + 32 * j;
                float v[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) v[q] = x[8 * j + q] * sc;
                uint4 hi, lo;
                split8(v, hi, lo);
                // samples 8c..8c+7 = (g0..g0+7, m) with g = i mod R, m = i / R
                const int i0 = 8 * c, m = i0 / R, g0 = i0 % R;
                const uint32_t off = mn_off(lf * R + g0, m);
                *reinterpret_cast<uint4*>(A1 + off) = hi;
                *reinterpret_cast<uint4*>(A1 + C::A1_BYTES / 2 + off) = lo;
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        // ---------------- pass 1 on the tensor cores
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < C::K1 / 16; ++ks) {
                const uint64_t ah = sdesc(a1 + ks * 4096, 1024, 2048);
                const uint64_t al = sdesc(a1 + C::A1_BYTES / 2 + ks * 4096, 1024, 2048);
                const uint64_t bh = sdesc(b1 + ks * 32, 16, 1024);
                const uint64_t bl = sdesc(b1 + C::B1_BYTES / 2 + ks * 32, 16, 1024);
                mma_f16(d1, ah, bh, ID, ks > 0);
                mma_f16(d1, ah, bl, ID, 1);
                mma_f16(d1, al, bh, ID, 1);
            }
            mma_commit(&mbar[0]);
        }
        if (!mbar_wait(&mbar[0], phase)) {
            if (lane == 0) atomicExch(abort_flag, 1);
        }
        __syncthreads();
        if (*abort_flag) {
            aborted = true;
            break;
        }
        fence_after();
        // ---------------- epilogue 1: twiddle, scale by 1/R, split -> A2 (row = this thread)
        {
            const int row = tid, lf = row / R, g = row % R;
            float y[C::NO];
#pragma unroll
            for (int cb = 0; cb < C::NO / 32; ++cb) {
                float t[32];
                tmem_ld32(d1 + lane_base + cb * 32, t);
#pragma unroll
                for (int i = 0; i < 32; ++i) y[cb * 32 + i] = t[i];
            }
            constexpr float inv_r = 1.0f / (float)R;
#pragma unroll
            for (int k1b = 0; k1b < R; k1b += 8) {
                float re[8], im[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int k1 = k1b + q;
                    const float2 w = TW[g * R + k1];
                    const float yr = y[2 * k1], yi = y[2 * k1 + 1];
                    re[q] = (yr * w.x - yi * w.y) * inv_r;
                    im[q] = (yr * w.y + yi * w.x) * inv_r;
                }
                uint4 hr, lr, hi_, li_;
                split8(re, hr, lr);
                split8(im, hi_, li_);
                const uint32_t or_ = mn_off(lf * R + k1b, g);
                const uint32_t oi_ = mn_off(lf * R + k1b, R + g);
                *reinterpret_cast<uint4*>(A2 + or_) = hr;
                *reinterpret_cast<uint4*>(A2 + C::A2_BYTES / 2 + or_) = lr;
                *reinterpret_cast<uint4*>(A2 + oi_) = hi_;
                *reinterpret_cast<uint4*>(A2 + C::A2_BYTES / 2 + oi_) = li_;
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        // ---------------- pass 2 on the tensor cores
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < C::K2 / 16; ++ks) {
                const uint64_t ah = sdesc(a2 + ks * 4096, 1024, 2048);
                const uint64_t al = sdesc(a2 + C::A2_BYTES / 2 + ks * 4096, 1024, 2048);
                const uint64_t bh = sdesc(b2 + ks * 32, 16, 1024);
                const uint64_t bl = sdesc(b2 + C::B2_BYTES / 2 + ks * 32, 16, 1024);
                mma_f16(d2, ah, bh, ID, ks > 0);
                mma_f16(d2, ah, bl, ID, 1);
                mma_f16(d2, al, bh, ID, 1);
            }
            mma_commit(&mbar[1]);
        }
        if (!mbar_wait(&mbar[1], phase)) {
            if (lane == 0) atomicExch(abort_flag, 1);
        }
        __syncthreads();
        if (*abort_flag) {
            aborted = true;
            break;
        }
        fence_after();
        // ---------------- epilogue 2: thread = (frame, k1) holds X[k1 + R k2]
        {
            const int row = tid, lf = row / R, k1 = row % R;
            const uint64_t f = f0 + lf;
            const bool act = f < a.frames;
            const float back = fscale[lf] * (float)R;  // undo both scalings (powers of two)
            float xs[C::NO];
#pragma unroll
            for (int cb = 0; cb < C::NO / 32; ++cb) {
                float t[32];
                tmem_ld32(d2 + lane_base + cb * 32, t);
#pragma unroll
                for (int i = 0; i < 32; ++i) xs[cb * 32 + i] = t[i];
            }
            if (act) {
                if constexpr (OUTK == OUT_HALF) {
                    float2* o2 = reinterpret_cast<float2*>(a.out);
#pragma unroll
                    for (int k2 = 0; k2 < R; ++k2) {
                        const int k = k1 + R * k2;
                        const float2 X = make_float2(xs[2 * k2] * back, xs[2 * k2 + 1] * back);
                        if (!a.dense) {
                            const uint64_t flat = f * (uint64_t)N + k;
                            if (flat < a.ohalf) __stcs(o2 + flat, X);
                        } else if (k <= N / 2) {
                            __stcs(o2 + f * (uint64_t)(N / 2 + 1) + k, X);
                        }
                    }
                } else {
#pragma unroll
                    for (int k2 = 0; k2 <= R / 2; ++k2) {
                        const int k = k1 + R * k2;
                        if (k > N / 2) continue;
                        const float xr = xs[2 * k2] * back, xi = xs[2 * k2 + 1] * back;
                        const float p = (OUTK == OUT_POWER_SERIAL) ? fabsf(xr) * 1.41421356237309505f
                                                                   : sqrtf(xr * xr + xi * xi);
                        if (!a.dense) {
                            float* rowp = a.out + f * (uint64_t)N;
                            __stcs(rowp + k, p);
                            if (k != 0 && k != N / 2) __stcs(rowp + (N - k), p);
                        } else {
                            __stcs(a.out + f * (uint64_t)(N / 2 + 1) + k, p);
                        }
                    }
                }
            }
        }
        fence_before();
        __syncthreads();
        fence_after();
        phase ^= 1u;
    }
    // ---------------- release tensor memory (every exit path)
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(C::TMEM_COLS));
    }
    if (aborted && tid == 0) *reinterpret_cast<volatile int*>(err) = 1;
}


// ============================================================ pipelined form
// Warp roles (448 threads, 14 warps):
//   warps 0-3   loaders: window, DC, per-frame scale, fp16 split -> A1[s]
//   warps 4-7   epilogue 1: D1 -> twiddle -> split -> A2[s]
//   warps 8-11  epilogue 2: D2 -> power / half-complex -> global memory
//   warp 12     one thread issues every MMA (both passes)
//   warp 13     one thread prefetches each tile's input span (TMA bulk copy)
// Operands (A1, A2), accumulators (D1, D2 in tensor memory) and the raw input
// are double-buffered, so the four stages work on different tiles at once.
// The DFT matrices and twiddles are built once per window size into global
// memory, already in the swizzled shared-memory image, and copied per CTA.
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* b)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(b))
                 : "memory");
}

// Waits for the phase of the given parity.  Gives up after one second of
// wall time (globaltimer) or as soon as another role of the CTA has given up.
__device__ __forceinline__ bool mbar_wait_t(uint64_t* mbar, uint32_t parity, const volatile int* abort_flag)
{
    const uint32_t a = smem_u32(mbar);
    uint64_t t0 = 0;
    for (uint32_t i = 0; i < (1u << 30); ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((i & 63) == 63) {
            if (abort_flag && *abort_flag) return false;
            uint64_t t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            if (t0 == 0) t0 = t;
            else if (t - t0 > 1000000000ull) return false;
        }
    }
    return false;
}

// Operand splits.  PM_FP16X2: x = hi + lo in fp16 (products hh + hl + lh);
// PM_BF16X2: the same in bf16 (8-bit significands: about 16 bits kept, for
// reference); PM_BF16X3: x = hi + mid + lo in bf16 (products hh, hm, mh, hl,
// lh, mm: about 24 bits, fp32-like).  Packed conversions, two values each.
enum { PM_FP16X2 = 1, PM_BF16X2 = 2, PM_BF16X3 = 3 };
template <int PM>
struct Split {
    static constexpr int PARTS = PM == PM_BF16X3 ? 3 : 2;
    static constexpr uint32_t FMT = PM == PM_FP16X2 ? 0u : 1u;  // tcgen05 kind::f16 operand format
    // p[k] receives part k of x[0..7], 8 halves in 16 bytes
    static __device__ __forceinline__ void split8(const float (&x)[8], uint4 (&p)[PARTS])
    {
        uint32_t w[PARTS][4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            float a = x[2 * i], b = x[2 * i + 1];
#pragma unroll
            for (int k = 0; k < PARTS; ++k) {
                if constexpr (PM == PM_FP16X2) {
                    const __half2 h = __floats2half2_rn(a, b);
                    const float2 f = __half22float2(h);
                    w[k][i] = *reinterpret_cast<const uint32_t*>(&h);
                    a -= f.x;
                    b -= f.y;
                } else {
                    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
                    const float2 f = __bfloat1622float2(h);
                    w[k][i] = *reinterpret_cast<const uint32_t*>(&h);
                    a -= f.x;
                    b -= f.y;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < PARTS; ++k) p[k] = make_uint4(w[k][0], w[k][1], w[k][2], w[k][3]);
    }
    static __device__ __forceinline__ void part1(float v, uint16_t (&o)[PARTS])
    {
#pragma unroll
        for (int k = 0; k < PARTS; ++k) {
            if constexpr (PM == PM_FP16X2) {
                const __half h = __float2half_rn(v);
                o[k] = __half_as_ushort(h);
                v -= __half2float(h);
            } else {
                const __nv_bfloat16 h = __float2bfloat16_rn(v);
                o[k] = __bfloat16_as_ushort(h);
                v -= __bfloat162float(h);
            }
        }
    }
};

// instruction descriptor of kind::f16 with the mode's operand format
template <int PM>
__host__ __device__ constexpr uint32_t idesc_pm(int M, int N)
{
    return idesc_f16(M, N) | (Split<PM>::FMT << 7) | (Split<PM>::FMT << 10);
}

template <int R, int PM>
struct Tc2Cfg {
    static constexpr int P = Split<PM>::PARTS;
    static constexpr int N = R * R;
    static constexpr int FPT = 128 / R;
    static constexpr int K1 = R, K2 = 2 * R, NO = 2 * R;
    static constexpr uint32_t RAW_BYTES = ((FPT * N + 64) * 4 + 1023) / 1024 * 1024;  // span of hop <= N
    static constexpr uint32_t A1_PART = (K1 / 8) * 2048;  // 128 rows, MN-major
    static constexpr uint32_t A2_PART = (K2 / 8) * 2048;
    static constexpr uint32_t A1_BYTES = P * A1_PART;
    static constexpr uint32_t A2_BYTES = P * A2_PART;
    static constexpr uint32_t B_PART = NO * 128;  // K <= 64: one 128-byte row per output column
    static constexpr uint32_t B1_BYTES = P * B_PART;
    static constexpr uint32_t B2_BYTES = P * B_PART;
    static constexpr uint32_t TW_BYTES = N * 8;
    static constexpr uint32_t TAB_BYTES = B1_BYTES + B2_BYTES + TW_BYTES;  // the prebuilt image
    // A2 double-buffered unless that overflows shared memory (bf16x3 at R = 32)
    static constexpr int NA2 = (2 * RAW_BYTES + 2 * A1_BYTES + 2 * A2_BYTES + TAB_BYTES + N * 4 + 2048) <= 227 * 1024
                                   ? 2
                                   : 1;
    static constexpr uint32_t OFF_RAW = 0;
    static constexpr uint32_t OFF_A1 = OFF_RAW + 2 * RAW_BYTES;
    static constexpr uint32_t OFF_A2 = OFF_A1 + 2 * A1_BYTES;
    static constexpr uint32_t OFF_B1 = OFF_A2 + NA2 * A2_BYTES;
    static constexpr uint32_t OFF_B2 = OFF_B1 + B1_BYTES;
    static constexpr uint32_t OFF_TW = OFF_B2 + B2_BYTES;
    static constexpr uint32_t OFF_WIN = OFF_TW + TW_BYTES;
    static constexpr uint32_t OFF_BAR = OFF_WIN + N * 4;
    static constexpr uint32_t OFF_MISC = OFF_BAR + 32 * 8;
    static constexpr uint32_t SMEM = OFF_MISC + 512 + 1024;
    static constexpr uint32_t TMEM_COLS = 4 * NO <= 128 ? 128 : 256;
    static_assert(TAB_BYTES % 16 == 0, "table image copied in 16-byte units");
    static_assert(SMEM <= 227 * 1024, "shared memory");
};

// prebuilt table images, one per window size and split mode
__device__ __align__(1024) unsigned char g_tc_tab16_1[Tc2Cfg<16, 1>::TAB_BYTES];
__device__ __align__(1024) unsigned char g_tc_tab16_2[Tc2Cfg<16, 2>::TAB_BYTES];
__device__ __align__(1024) unsigned char g_tc_tab16_3[Tc2Cfg<16, 3>::TAB_BYTES];
__device__ __align__(1024) unsigned char g_tc_tab32_1[Tc2Cfg<32, 1>::TAB_BYTES];
__device__ __align__(1024) unsigned char g_tc_tab32_2[Tc2Cfg<32, 2>::TAB_BYTES];
__device__ __align__(1024) unsigned char g_tc_tab32_3[Tc2Cfg<32, 3>::TAB_BYTES];

// B1: rows 2k1 (re), 2k1+1 (im) of the real-input r-point DFT, K = m.
// B2: the complex r-point DFT as a real matrix, K = g (re part, k < R) and
// g (im part, k >= R).  TW: W_N^{g k1} / R, stored [k1][g].
template <int R, int PM>
__global__ void build_tc_tables_kernel(unsigned char* img)
{
    using C = Tc2Cfg<R, PM>;
    using S = Split<PM>;
    unsigned char* B1 = img;
    unsigned char* B2 = img + C::B1_BYTES;
    float2* TW = reinterpret_cast<float2*>(img + C::B1_BYTES + C::B2_BYTES);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (int e = tid; e < C::NO * C::K1; e += nth) {
        const int row = e / C::K1, m = e % C::K1, k1 = row >> 1;
        double sn, cs;
        sincospi(2.0 * (double)((m * k1) % R) / (double)R, &sn, &cs);
        uint16_t pt[S::PARTS];
        S::part1((row & 1) ? (float)(-sn) : (float)cs, pt);
        for (int k = 0; k < S::PARTS; ++k) *reinterpret_cast<uint16_t*>(B1 + k * C::B_PART + k_off(row, m)) = pt[k];
    }
    for (int e = tid; e < C::NO * C::K2; e += nth) {
        const int row = e / C::K2, k = e % C::K2, k2 = row >> 1, g = k % R;
        double sn, cs;
        sincospi(2.0 * (double)((g * k2) % R) / (double)R, &sn, &cs);
        // (yr + i yi)(c - i s): re = yr c + yi s, im = yi c - yr s
        float w;
        if ((row & 1) == 0) w = (k < R) ? (float)cs : (float)sn;
        else w = (k < R) ? (float)(-sn) : (float)cs;
        uint16_t pt[S::PARTS];
        S::part1(w, pt);
        for (int q = 0; q < S::PARTS; ++q) *reinterpret_cast<uint16_t*>(B2 + q * C::B_PART + k_off(row, k)) = pt[q];
    }
    for (int e = tid; e < C::N; e += nth) {
        const int k1 = e / R, g = e % R;
        double sn, cs;
        sincospi(2.0 * (double)((g * k1) % C::N) / (double)C::N, &sn, &cs);
        // 1/R is a power of two: folding it in changes no rounding
        TW[e] = make_float2((float)cs / (float)R, (float)(-sn) / (float)R);
    }
}

enum { B_RAW_FULL = 0, B_RAW_EMPTY = 2, B_A1_FULL = 4, B_A1_EMPTY = 6, B_D1_FULL = 8, B_D1_EMPTY = 10,
       B_A2_FULL = 12, B_A2_EMPTY = 14, B_D2_FULL = 16, B_D2_EMPTY = 18, B_FIN = 20, B_COUNT = 21 };

constexpr int kTc2Threads = 448;

template <int R, int OUTK, int PM>
__global__ void __launch_bounds__(kTc2Threads, 1)
    stft_tc2_kernel(const FusedArgs a, const unsigned char* __restrict__ tab, volatile int* err, int test_stall)
{
    using C = Tc2Cfg<R, PM>;
    using S = Split<PM>;
    constexpr int P = C::P;
    constexpr int N = C::N, FPT = C::FPT;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float* RAW = reinterpret_cast<float*>(sm + C::OFF_RAW);
    unsigned char* A1 = sm + C::OFF_A1;
    unsigned char* A2 = sm + C::OFF_A2;
    const float2* TW = reinterpret_cast<const float2*>(sm + C::OFF_TW);
    float* WIN = reinterpret_cast<float*>(sm + C::OFF_WIN);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + C::OFF_BAR);
    unsigned char* misc = sm + C::OFF_MISC;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(misc);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(misc + 8);
    uint64_t* raw_base = reinterpret_cast<uint64_t*>(misc + 16);  // [2]
    uint64_t* raw_end = reinterpret_cast<uint64_t*>(misc + 32);   // [2]
    // per-frame scales travel with the tile: loaders -> sA -> (MMA thread) sB
    // -> (epilogue 1) sC -> (MMA thread) sD -> epilogue 2; each copy happens
    // between the wait on a stage's "full" barrier and the release of its
    // "empty" one, so no slot is rewritten while still being read
    float* sA = reinterpret_cast<float*>(misc + 64);
    float* sB = sA + 2 * FPT;
    float* sC = sB + 2 * FPT;
    float* sD = sC + 2 * FPT;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(&bar[B_RAW_FULL + s], 1);
            mbar_init(&bar[B_RAW_EMPTY + s], 128);
            mbar_init(&bar[B_A1_FULL + s], 128);
            mbar_init(&bar[B_A1_EMPTY + s], 1);
            mbar_init(&bar[B_D1_FULL + s], 2);  // MMA completion + the thread's copy of the scales
            mbar_init(&bar[B_D1_EMPTY + s], 128);
            mbar_init(&bar[B_A2_FULL + s], 128);
            mbar_init(&bar[B_A2_EMPTY + s], 1);
            mbar_init(&bar[B_D2_FULL + s], 2);
            mbar_init(&bar[B_D2_EMPTY + s], 128);
        }
        mbar_init(&bar[B_FIN], 1);
        *abort_flag = 0;
    }
    if (warp == 12) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(C::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    {
        const uint4* src = reinterpret_cast<const uint4*>(tab);
        uint4* dst = reinterpret_cast<uint4*>(sm + C::OFF_B1);
        for (int e = tid; e < (int)(C::TAB_BYTES / 16); e += kTc2Threads) dst[e] = src[e];
        // window stored so that the float4 a lane needs for (j, h) sits at
        // WIN[((2 j + h) * 32 + lane) * 4]: one warp-wide load reads 512
        // contiguous bytes (lane owns samples 8 (lane + 32 j) .. + 7)
        for (int e = tid; e < N; e += kTc2Threads) {
            const int c = e >> 3, h = (e >> 2) & 1, k = e & 3, ln = c & 31, j = c >> 5;
            WIN[((2 * j + h) * 32 + ln) * 4 + k] = a.win ? a.win[e] : 1.0f;
        }
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    constexpr uint32_t ID = idesc_pm<PM>(128, C::NO);
    // products kept, as (A part, B part): hi*hi first, then the cross terms
    constexpr int NPROD = P == 3 ? 6 : 3;
    constexpr int PA[6] = {0, 0, 1, 0, 2, 1};
    constexpr int PB[6] = {0, 1, 0, 2, 0, 1};

    const uint64_t ntiles = (a.frames + FPT - 1) / FPT;
    const uint64_t cnt = blockIdx.x < ntiles ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    auto tile_of = [&](uint64_t i) { return blockIdx.x + i * gridDim.x; };
    auto give_up = [&]() {
        *abort_flag = 1;
        *err = 1;
    };
    // Samples are addressed from xb = a.x rounded down to 16 bytes (the same
    // 16-byte block, so still inside the caller's allocation): sample gi sits
    // at xb[gi + mis].  Every bulk copy then starts and ends on 16 bytes.
    const uint32_t mis = (uint32_t)((reinterpret_cast<uintptr_t>(a.x) & 15u) >> 2);
    const float* xb = a.x - mis;

    if (warp == 13) {
        // ---------------- producer: one bulk copy of each tile's input span
        if (lane == 0) {
            uint32_t issued[2] = {0, 0};
            for (uint64_t i = 0; i < cnt && !*abort_flag; ++i) {
                const int r = (int)(i & 1);
                const uint32_t use = (uint32_t)(i >> 1);
                if (i >= 2 && !mbar_wait_t(&bar[B_RAW_EMPTY + r], (use - 1) & 1, abort_flag)) {
                    give_up();
                    break;
                }
                const uint64_t f0 = tile_of(i) * FPT;
                const uint64_t nf = (a.frames - f0) < (uint64_t)FPT ? (a.frames - f0) : (uint64_t)FPT;
                // virtual (xb-relative) span [a0, e16) of the tile, 16-byte granular;
                // the loaders read the few samples past e16 from global memory
                const uint64_t s0 = f0 * a.hop + mis;
                const uint64_t a0 = s0 & ~(uint64_t)3;
                uint64_t send = (f0 + nf - 1) * a.hop + N;
                if (send > a.n) send = a.n;
                send += mis;
                const uint64_t e16 = send > a0 ? a0 + ((send - a0) & ~(uint64_t)3) : a0;
                raw_base[r] = a0;
                raw_end[r] = e16;
                const uint32_t bytes = (uint32_t)((e16 - a0) * 4);
                if (test_stall && i == 0) continue;  // test hook: nothing ever completes this phase
                if (bytes) {
                    mbar_expect_tx(&bar[B_RAW_FULL + r], bytes);
                    bulk_g2s(RAW + r * (C::RAW_BYTES / 4), xb + a0, bytes, &bar[B_RAW_FULL + r]);
                } else {
                    mbar_arrive(&bar[B_RAW_FULL + r]);
                }
                ++issued[r];
            }
            // no copy may still be landing in shared memory when the CTA exits
            for (int r = 0; r < 2; ++r)
                if (issued[r]) mbar_wait_t(&bar[B_RAW_FULL + r], (issued[r] - 1) & 1, nullptr);
        }
    } else if (warp == 12) {
        // ---------------- MMA issuer: MMA1(i), then MMA2(i-1)
        if (lane == 0) {
            const uint32_t b1 = smem_u32(sm + C::OFF_B1), b2 = smem_u32(sm + C::OFF_B2);
            for (uint64_t i = 0; i <= cnt && !*abort_flag; ++i) {
                if (i < cnt) {
                    const int s = (int)(i & 1);
                    const uint32_t use = (uint32_t)(i >> 1);
                    if (!mbar_wait_t(&bar[B_A1_FULL + s], use & 1, abort_flag) ||
                        (i >= 2 && !mbar_wait_t(&bar[B_D1_EMPTY + s], (use - 1) & 1, abort_flag))) {
                        give_up();
                        break;
                    }
                    for (int q = 0; q < FPT; ++q) sB[s * FPT + q] = sA[s * FPT + q];
                    fence_after();
                    const uint32_t a1 = smem_u32(A1 + s * C::A1_BYTES);
                    const uint32_t d1 = tmem + s * C::NO;
#pragma unroll
                    for (int ks = 0; ks < C::K1 / 16; ++ks) {
#pragma unroll
                        for (int q = 0; q < NPROD; ++q) {
                            const uint64_t ad = sdesc(a1 + PA[q] * C::A1_PART + ks * 4096, 1024, 2048);
                            const uint64_t bd = sdesc(b1 + PB[q] * C::B_PART + ks * 32, 16, 1024);
                            mma_f16(d1, ad, bd, ID, (ks > 0 || q > 0) ? 1u : 0u);
                        }
                    }
                    mma_commit(&bar[B_A1_EMPTY + s]);
                    mma_commit(&bar[B_D1_FULL + s]);
                    mbar_arrive(&bar[B_D1_FULL + s]);
                }
                if (i >= 1) {
                    const uint64_t j = i - 1;
                    const int s = (int)(j & 1);
                    const uint32_t use = (uint32_t)(j >> 1);
                    const int s2 = (int)(j % C::NA2);  // A2 slot
                    const uint32_t use2 = (uint32_t)(j / C::NA2);
                    if (!mbar_wait_t(&bar[B_A2_FULL + s2], use2 & 1, abort_flag) ||
                        (j >= 2 && !mbar_wait_t(&bar[B_D2_EMPTY + s], (use - 1) & 1, abort_flag))) {
                        give_up();
                        break;
                    }
                    for (int q = 0; q < FPT; ++q) sD[s * FPT + q] = sC[s2 * FPT + q];
                    fence_after();
                    const uint32_t a2 = smem_u32(A2 + s2 * C::A2_BYTES);
                    const uint32_t d2 = tmem + 2 * C::NO + s * C::NO;
#pragma unroll
                    for (int ks = 0; ks < C::K2 / 16; ++ks) {
#pragma unroll
                        for (int q = 0; q < NPROD; ++q) {
                            const uint64_t ad = sdesc(a2 + PA[q] * C::A2_PART + ks * 4096, 1024, 2048);
                            const uint64_t bd = sdesc(b2 + PB[q] * C::B_PART + ks * 32, 16, 1024);
                            mma_f16(d2, ad, bd, ID, (ks > 0 || q > 0) ? 1u : 0u);
                        }
                    }
                    mma_commit(&bar[B_A2_EMPTY + s2]);
                    mma_commit(&bar[B_D2_FULL + s]);
                    mbar_arrive(&bar[B_D2_FULL + s]);
                }
            }
            // every MMA of this CTA has finished before tensor memory is released
            mma_commit(&bar[B_FIN]);
            mbar_wait_t(&bar[B_FIN], 0, nullptr);
        }
    } else if (warp < 4) {
        // ---------------- loaders: window, DC, scale, split -> A1[s]
        for (uint64_t i = 0; i < cnt; ++i) {
            const int s = (int)(i & 1);
            const uint32_t use = (uint32_t)(i >> 1);
            bool ok = mbar_wait_t(&bar[B_RAW_FULL + s], use & 1, abort_flag);
            if (ok && i >= 2) ok = mbar_wait_t(&bar[B_A1_EMPTY + s], (use - 1) & 1, abort_flag);
            // one decision per warp: the shuffles below need every lane
            if (!__all_sync(0xffffffffu, ok && !*abort_flag)) {
                give_up();
                break;
            }
            const uint64_t f0 = tile_of(i) * FPT;
            const uint64_t a0 = raw_base[s], e16 = raw_end[s];
            const float* raw = RAW + s * (C::RAW_BYTES / 4);
            unsigned char* a1 = A1 + s * C::A1_BYTES;
            for (int lf = warp; lf < FPT; lf += 4) {
                const uint64_t f = f0 + lf;
                const bool act = f < a.frames;
                const uint64_t sb = f * a.hop + mis;  // virtual start of the frame
                float x[N / 32];
                // fast: the whole frame is staged and starts on a 16-byte word
                const bool fast = act && sb + N <= e16 && ((sb - a0) & 3) == 0;
#pragma unroll
                for (int j = 0; j < N / 256; ++j) {  // lane owns samples [8c, 8c+8), c = lane + 32 j
                    const int c = lane + 32 * j;
                    if (fast) {
                        const float4 p = *reinterpret_cast<const float4*>(raw + (sb - a0) + 8 * c);
                        const float4 q = *reinterpret_cast<const float4*>(raw + (sb - a0) + 8 * c + 4);
                        x[8 * j + 0] = p.x; x[8 * j + 1] = p.y; x[8 * j + 2] = p.z; x[8 * j + 3] = p.w;
                        x[8 * j + 4] = q.x; x[8 * j + 5] = q.y; x[8 * j + 6] = q.z; x[8 * j + 7] = q.w;
                    } else {
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const uint64_t vi = sb + 8 * c + q;  // sample vi - mis
                            float v = 0.0f;
                            if (act && vi < a.n + mis) v = vi < e16 ? raw[vi - a0] : xb[vi];
                            x[8 * j + q] = v;
                        }
                    }
                }
                float sum = 0.0f;
#pragma unroll
                for (int j = 0; j < N / 256; ++j) {
                    const float4 w0 = *reinterpret_cast<const float4*>(WIN + ((2 * j) * 32 + lane) * 4);
                    const float4 w1 = *reinterpret_cast<const float4*>(WIN + ((2 * j + 1) * 32 + lane) * 4);
                    const float wv[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        x[8 * j + q] *= wv[q];
                        sum += x[8 * j + q];
                    }
                }
                if (a.remove_dc) {
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
                    const float mean = sum * (1.0f / (float)N);
#pragma unroll
                    for (int q = 0; q < N / 32; ++q) x[q] -= mean;
                }
                float mx = 0.0f;
#pragma unroll
                for (int q = 0; q < N / 32; ++q) mx = fmaxf(mx, fabsf(x[q]));
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                int e2 = 0;
                if (mx > 0.0f) frexpf(mx, &e2);  // mx in [2^(e2-1), 2^e2)
                const float sc = ldexpf(1.0f, 14 - e2);
                if (lane == 0) sA[s * FPT + lf] = ldexpf(1.0f, e2 - 14);
#pragma unroll
                for (int j = 0; j < N / 256; ++j) {
                    const int c = lane + 32 * j;
                    float v[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) v[q] = x[8 * j + q] * sc;
                    uint4 pt[P];
                    S::split8(v, pt);
                    // samples 8c..8c+7 = (g0..g0+7, m) with g = i mod R, m = i / R
                    const int i0 = 8 * c, m = i0 / R, g0 = i0 % R;
                    const uint32_t dst = mn_off(lf * R + g0, m);
#pragma unroll
                    for (int k = 0; k < P; ++k) *reinterpret_cast<uint4*>(a1 + k * C::A1_PART + dst) = pt[k];
                }
            }
            mbar_arrive(&bar[B_RAW_EMPTY + s]);
            fence_async_smem();
            mbar_arrive(&bar[B_A1_FULL + s]);
        }
    } else if (warp < 8) {
        // ---------------- epilogue 1: row = TMEM lane = (frame, g)
        const int row = tid - 128, lf = row / R, g = row % R;
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        for (uint64_t i = 0; i < cnt; ++i) {
            const int s = (int)(i & 1);
            const uint32_t use = (uint32_t)(i >> 1);
            const bool ok = mbar_wait_t(&bar[B_D1_FULL + s], use & 1, abort_flag);
            if (!__all_sync(0xffffffffu, ok && !*abort_flag)) {
                give_up();
                break;
            }
            fence_after();
            const float scale = sB[s * FPT + lf];
            const int s2 = (int)(i % C::NA2);  // A2 slot
            const uint32_t use2 = (uint32_t)(i / C::NA2);
            const bool ok2 = i < (uint64_t)C::NA2 || mbar_wait_t(&bar[B_A2_EMPTY + s2], (use2 - 1) & 1, abort_flag);
            if (!__all_sync(0xffffffffu, ok2)) {
                give_up();
                break;
            }
            if (g == 0) sC[s2 * FPT + lf] = scale;
            unsigned char* a2 = A2 + s2 * C::A2_BYTES;
            // eight k1 (sixteen accumulator columns) per step, the loop kept
            // rolled: the four warp roles run different code at the same time
            // and instruction fetch was what limited the kernel
#pragma unroll 1
            for (int k1b = 0; k1b < R; k1b += 8) {
                float t[16];
                tmem_ld16(tmem + s * C::NO + lane_base + 2 * k1b, t);
                float re[8], im[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float2 w = TW[(k1b + q) * R + g];  // W_N^{g k1} / R
                    const float yr = t[2 * q], yi = t[2 * q + 1];
                    re[q] = yr * w.x - yi * w.y;
                    im[q] = yr * w.y + yi * w.x;
                }
                uint4 pr[P], pi[P];
                S::split8(re, pr);
                S::split8(im, pi);
                const uint32_t or_ = mn_off(lf * R + k1b, g);
                const uint32_t oi_ = mn_off(lf * R + k1b, R + g);
#pragma unroll
                for (int k = 0; k < P; ++k) {
                    *reinterpret_cast<uint4*>(a2 + k * C::A2_PART + or_) = pr[k];
                    *reinterpret_cast<uint4*>(a2 + k * C::A2_PART + oi_) = pi[k];
                }
            }
            fence_before();
            mbar_arrive(&bar[B_D1_EMPTY + s]);
            fence_async_smem();
            mbar_arrive(&bar[B_A2_FULL + s2]);
        }
    } else {
        // ---------------- epilogue 2: row = TMEM lane = (frame, k1), holds X[k1 + R k2]
        const int row = tid - 256, lf = row / R, k1 = row % R;
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        for (uint64_t j = 0; j < cnt; ++j) {
            const int s = (int)(j & 1);
            const uint32_t use = (uint32_t)(j >> 1);
            const bool ok = mbar_wait_t(&bar[B_D2_FULL + s], use & 1, abort_flag);
            if (!__all_sync(0xffffffffu, ok && !*abort_flag)) {
                give_up();
                break;
            }
            fence_after();
            const float back = sD[s * FPT + lf] * (float)R;  // undo both scalings (powers of two)
            const uint64_t f = tile_of(j) * FPT + lf;
            const bool act = f < a.frames;
            // eight k2 per step, rolled (see epilogue 1); the accumulator loads
            // run on every lane (they are warp-collective), the stores only
            // for rows of real frames
            constexpr int K2END = OUTK == OUT_HALF ? R : R / 2 + 1;
#pragma unroll 1
            for (int k2b = 0; k2b < K2END; k2b += 8) {
                float t[16];
                tmem_ld16(tmem + 2 * C::NO + s * C::NO + lane_base + 2 * k2b, t);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int k2 = k2b + q;
                    if (!act || k2 >= K2END) break;
                    const int k = k1 + R * k2;
                    const float xr = t[2 * q] * back, xi = t[2 * q + 1] * back;
                    if constexpr (OUTK == OUT_HALF) {
                        float2* o2 = reinterpret_cast<float2*>(a.out);
                        const float2 X = make_float2(xr, xi);
                        if (!a.dense) {
                            const uint64_t flat = f * (uint64_t)N + k;
                            if (flat < a.ohalf) __stcs(o2 + flat, X);
                        } else if (k <= N / 2) {
                            __stcs(o2 + f * (uint64_t)(N / 2 + 1) + k, X);
                        }
                    } else {
                        if (k > N / 2) continue;
                        const float p = (OUTK == OUT_POWER_SERIAL) ? fabsf(xr) * 1.41421356237309505f
                                                                   : sqrtf(xr * xr + xi * xi);
                        if (!a.dense) {
                            float* rowp = a.out + f * (uint64_t)N;
                            __stcs(rowp + k, p);
                            if (k != 0 && k != N / 2) __stcs(rowp + (N - k), p);
                        } else {
                            __stcs(a.out + f * (uint64_t)(N / 2 + 1) + k, p);
                        }
                    }
                }
            }
            fence_before();
            mbar_arrive(&bar[B_D2_EMPTY + s]);
        }
    }
    __syncwarp();
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 12) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(C::TMEM_COLS));
    }
}

// ============================================================ generic form
// Windows N = P * Q with P >= Q: 512 = 32 x 16, 2048 = 64 x 32, 4096 = 64 x 64.
// The same four-step DFT as above with n = g + Q m and k = k1 + P k2:
//   pass 1  Y[g][k1] = sum_m y[g + Q m] W_P^{m k1}   GEMM rows (frame, g), K = m
//   twiddle Y[g][k1] *= W_N^{g k1} / P
//   pass 2  X[k1 + P k2] = sum_g Y[g][k1] W_Q^{g k2} GEMM rows (frame, k1), K = re/im of g
// A tile is 128 / Q frames: 128 pass-1 rows and P / Q blocks of 128 pass-2
// rows.  One CTA of 128 threads works one tile at a time (thread i owns TMEM
// lane i): load + split, pass 1, epilogue 1, pass 2, epilogue 2.  A1 and A2
// share one region (pass 1 has completed before A2 is written); B2 is stored
// as 64-wide K panels; the twiddles come from a two-level table
// W_N^e = lo[e & 63] * hi[e >> 6].  Every operand split of the pipelined form
// is available where its operands fit in shared memory (the bf16 hi/mid/lo
// split at 4096 does not: about 240 KB).
template <int P, int Q, int PM>
struct TcgCfg {
    static constexpr int N = P * Q;
    static constexpr int PARTS = Split<PM>::PARTS;
    static constexpr int FPT = 128 / Q;         // frames per tile
    static constexpr int MB = P / Q;            // pass-2 blocks of 128 rows
    static constexpr int K1 = P, NO1 = 2 * P;   // pass 1
    static constexpr int K2 = 2 * Q, NO2 = 2 * Q;  // pass 2
    static constexpr int KP2 = (K2 + 63) / 64;  // B2 panels of 64 K
    static constexpr uint32_t A1_PART = (K1 / 8) * 2048;  // 128 rows, MN-major
    static constexpr uint32_t A2_PART_FULL = (K2 / 8) * 2048;
    static constexpr uint32_t A1_BYTES = PARTS * A1_PART;
    static constexpr uint32_t B1_PART = NO1 * 128;  // K1 <= 64: one 128-byte row per output column
    static constexpr uint32_t B2_PANEL = NO2 * 128;
    static constexpr uint32_t B2_PART = KP2 * B2_PANEL;
    static constexpr uint32_t B1_BYTES = PARTS * B1_PART;
    static constexpr uint32_t B2_BYTES = PARTS * B2_PART;
    // Pass 2 in two halves of K (real parts, then imaginary parts, through one
    // A2 buffer of half the size) where the whole A2 does not fit beside the
    // DFT matrices: 4096 = 64 x 64 with bf16 hi/mid/lo operands (242 KB whole)
    static constexpr uint32_t A2_WHOLE_BYTES = MB * PARTS * A2_PART_FULL;
    static constexpr uint32_t SMEM_WHOLE = (A1_BYTES > A2_WHOLE_BYTES ? A1_BYTES : A2_WHOLE_BYTES) + B1_BYTES +
                                           B2_BYTES + 128 * 8 + 256 + 1024;
    static constexpr int KH = (SMEM_WHOLE > 227 * 1024 && MB == 1 && Q % 16 == 0) ? 2 : 1;
    static constexpr uint32_t A2_PART = A2_PART_FULL / KH;  // one K half (or the whole K)
    static constexpr uint32_t A2_BLOCK = PARTS * A2_PART;
    static constexpr uint32_t A2_BYTES = MB * A2_BLOCK;
    static constexpr uint32_t A_BYTES = A1_BYTES > A2_BYTES ? A1_BYTES : A2_BYTES;
    static constexpr uint32_t OFF_A = 0;
    static constexpr uint32_t OFF_B1 = OFF_A + A_BYTES;
    static constexpr uint32_t OFF_B2 = OFF_B1 + B1_BYTES;
    static constexpr uint32_t OFF_TW = OFF_B2 + B2_BYTES;  // 128 float2: lo[64], hi[64]
    static constexpr uint32_t OFF_MISC = OFF_TW + 128 * 8;
    static constexpr uint32_t SMEM = OFF_MISC + 256 + 1024;  // + slack to 1024-align the base
    static constexpr uint32_t TMEM_USED = NO1 + MB * NO2;  // D1, then the D2 blocks
    static constexpr uint32_t TMEM_COLS = TMEM_USED <= 128 ? 128 : 256;
    static constexpr bool FITS = SMEM <= 227 * 1024;
    static_assert(K1 <= 64 && P >= Q && P % Q == 0 && 128 % Q == 0 && N <= 4096, "shapes");
    static_assert(TMEM_USED <= 256, "tensor memory");
};

template <int P, int Q, int OUTK, int PM>
__global__ void __launch_bounds__(128, 1) stft_tcg_kernel(const FusedArgs a, int* err)
{
    using C = TcgCfg<P, Q, PM>;
    using S = Split<PM>;
    static_assert(C::FITS, "shared memory");
    constexpr int N = C::N, FPT = C::FPT, PARTS = C::PARTS, MB = C::MB;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* A = sm + C::OFF_A;
    unsigned char* B1 = sm + C::OFF_B1;
    unsigned char* B2 = sm + C::OFF_B2;
    float2* TWL = reinterpret_cast<float2*>(sm + C::OFF_TW);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + C::OFF_MISC);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + C::OFF_MISC + 16);
    int* abort_flag = reinterpret_cast<int*>(sm + C::OFF_MISC + 24);
    float* fscale = reinterpret_cast<float*>(sm + C::OFF_MISC + 32);  // FPT (<= 8) entries

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // ---------------- set-up: barriers, tensor memory, DFT matrices, twiddles
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar[1])));
        *abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"(C::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    // B1: rows 2k1 (re), 2k1+1 (im) of the real-input P-point DFT, K = m
    for (int e = tid; e < C::NO1 * C::K1; e += 128) {
        const int row = e / C::K1, m = e % C::K1, k1 = row >> 1;
        double sn, cs;
        sincospi(2.0 * (double)((m * k1) % P) / (double)P, &sn, &cs);
        uint16_t pt[PARTS];
        S::part1((row & 1) ? (float)(-sn) : (float)cs, pt);
#pragma unroll
        for (int k = 0; k < PARTS; ++k) *reinterpret_cast<uint16_t*>(B1 + k * C::B1_PART + k_off(row, m)) = pt[k];
    }
    // B2: the complex Q-point DFT as a real matrix, K = g (re part, k < Q) and g (im part, k >= Q)
    for (int e = tid; e < C::NO2 * C::K2; e += 128) {
        const int row = e / C::K2, k = e % C::K2, k2 = row >> 1, g = k % Q;
        double sn, cs;
        sincospi(2.0 * (double)((g * k2) % Q) / (double)Q, &sn, &cs);
        // (yr + i yi)(c - i s): re = yr c + yi s, im = yi c - yr s
        float w;
        if ((row & 1) == 0) w = (k < Q) ? (float)cs : (float)sn;
        else w = (k < Q) ? (float)(-sn) : (float)cs;
        uint16_t pt[PARTS];
        S::part1(w, pt);
        const uint32_t off = (k >> 6) * C::B2_PANEL + k_off(row, k & 63);
#pragma unroll
        for (int q = 0; q < PARTS; ++q) *reinterpret_cast<uint16_t*>(B2 + q * C::B2_PART + off) = pt[q];
    }
    // two-level twiddles: W_N^e for e < 64, then W_N^(64 h) for h < 64
    for (int e = tid; e < 128; e += 128) {
        const int j = e < 64 ? e : (e - 64) * 64;
        double sn, cs;
        sincospi(2.0 * (double)(j % N) / (double)N, &sn, &cs);
        TWL[e] = make_float2((float)cs, (float)(-sn));
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t d1 = tmem, d2 = tmem + C::NO1;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    constexpr uint32_t ID1 = idesc_pm<PM>(128, C::NO1);
    constexpr uint32_t ID2 = idesc_pm<PM>(128, C::NO2);
    constexpr int NPROD = PARTS == 3 ? 6 : 3;
    constexpr int PA[6] = {0, 0, 1, 0, 2, 1};
    constexpr int PB[6] = {0, 1, 0, 2, 0, 1};
    const uint32_t sa = smem_u32(A), sb1 = smem_u32(B1), sb2 = smem_u32(B2);

    const uint64_t ntiles = (a.frames + FPT - 1) / FPT;
    uint32_t phase = 0, phase1 = 0;  // parities of the pass-1 and pass-2 barriers
    bool aborted = false;
    for (uint64_t tile = blockIdx.x; tile < ntiles && !aborted; tile += gridDim.x) {
        const uint64_t f0 = tile * FPT;
        // ---------------- load + window + DC + scale + split -> A1 (one warp per frame)
        for (int lf = warp; lf < FPT; lf += 4) {
            const uint64_t f = f0 + lf;
            const bool act = f < a.frames;
            const uint64_t s0 = f * a.hop;
            // the lane's 8 windowed samples [8c, 8c+8): two float4 loads of
            // samples and of window when the frame lies inside the signal and
            // both start on 16 bytes, else one bounded load each
            const bool vec = act && s0 + N <= a.n && a.win &&
                             ((reinterpret_cast<uintptr_t>(a.x + s0) | reinterpret_cast<uintptr_t>(a.win)) & 15) == 0;
            auto load8 = [&](int c, float (&v)[8]) {
                if (vec) {
                    const float4* xp = reinterpret_cast<const float4*>(a.x + s0 + 8 * c);
                    const float4* wp = reinterpret_cast<const float4*>(a.win + 8 * c);
                    const float4 x0 = xp[0], x1 = xp[1], w0 = wp[0], w1 = wp[1];
                    v[0] = x0.x * w0.x;
                    v[1] = x0.y * w0.y;
                    v[2] = x0.z * w0.z;
                    v[3] = x0.w * w0.w;
                    v[4] = x1.x * w1.x;
                    v[5] = x1.y * w1.y;
                    v[6] = x1.z * w1.z;
                    v[7] = x1.w * w1.w;
                } else {
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int i = 8 * c + q;
                        const uint64_t gi = s0 + i;
                        float t = (act && gi < a.n) ? a.x[gi] : 0.0f;
                        if (a.win) t *= a.win[i];
                        v[q] = t;
                    }
                }
            };
            // first read: sum, minimum and maximum of the windowed frame
            float sum = 0.0f, mn = 0.0f, mx = 0.0f;
            for (int j = 0; j < N / 256; ++j) {  // lane owns samples [8c, 8c+8), c = lane + 32 j
                float v[8];
                load8(lane + 32 * j, v);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    sum += v[q];
                    mn = fminf(mn, v[q]);
                    mx = fmaxf(mx, v[q]);
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sum += __shfl_xor_sync(0xffffffffu, sum, o);
                mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
                mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            }
            const float mean = a.remove_dc ? sum * (1.0f / (float)N) : 0.0f;
            const float peak = fmaxf(mx - mean, mean - mn);
            int e2 = 0;
            if (peak > 0.0f) frexpf(peak, &e2);  // peak in [2^(e2-1), 2^e2)
            const float sc = ldexpf(1.0f, 14 - e2);
            if (lane == 0) fscale[lf] = ldexpf(1.0f, e2 - 14);
            // second read (through L1): centre, scale, split
            for (int j = 0; j < N / 256; ++j) {
                const int c = lane + 32 * j;
                float v[8];
                load8(c, v);
#pragma unroll
                for (int q = 0; q < 8; ++q) v[q] = (v[q] - mean) * sc;
                uint4 pp[PARTS];
                S::split8(v, pp);
                // samples 8c .. 8c+7 = (g0 .. g0+7, m) with g = i mod Q, m = i / Q
                const int i0 = 8 * c, m = i0 / Q, g0 = i0 % Q;
                const uint32_t off = mn_off(lf * Q + g0, m);
#pragma unroll
                for (int k = 0; k < PARTS; ++k) *reinterpret_cast<uint4*>(A + k * C::A1_PART + off) = pp[k];
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        // ---------------- pass 1 on the tensor cores
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < C::K1 / 16; ++ks) {
#pragma unroll
                for (int pr = 0; pr < NPROD; ++pr) {
                    const uint64_t ad = sdesc(sa + PA[pr] * C::A1_PART + ks * 4096, 1024, 2048);
                    const uint64_t bd = sdesc(sb1 + PB[pr] * C::B1_PART + ks * 32, 16, 1024);
                    mma_f16(d1, ad, bd, ID1, (ks > 0 || pr > 0) ? 1u : 0u);
                }
            }
            mma_commit(&mbar[0]);
        }
        if (!mbar_wait(&mbar[0], phase)) {
            if (lane == 0) atomicExch(abort_flag, 1);
        }
        __syncthreads();
        if (*abort_flag) {
            aborted = true;
            break;
        }
        fence_after();
        // ---------------- epilogue 1 and pass 2, over the K halves of pass 2 (one
        // half, the whole K, unless the whole A2 does not fit)
#pragma unroll 1
        for (int h = 0; h < C::KH; ++h) {
            if (h > 0) {
                // the previous half's MMAs have read A2 (their commit arrived)
                fence_before();
                __syncthreads();
                fence_after();
            }
            // epilogue 1: twiddle, scale by 1/P, split -> A2 (row = this thread)
            {
                const int lf = tid / Q, g = tid % Q;
                constexpr float inv_p = 1.0f / (float)P;
#pragma unroll 1
                for (int k1b = 0; k1b < P; k1b += 8) {
                    float t[16];
                    tmem_ld16(d1 + lane_base + 2 * k1b, t);
                    float re[8], im[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int e = (g * (k1b + q)) & (N - 1);
                        const float2 w = cmul2(TWL[e & 63], TWL[64 + (e >> 6)]);
                        const float yr = t[2 * q], yi = t[2 * q + 1];
                        re[q] = (yr * w.x - yi * w.y) * inv_p;
                        im[q] = (yr * w.y + yi * w.x) * inv_p;
                    }
                    const int row2 = lf * P + k1b;  // 8 consecutive pass-2 rows, one block
                    unsigned char* blk = A + (row2 >> 7) * C::A2_BLOCK;
                    if (C::KH == 1 || h == 0) {
                        uint4 pr_[PARTS];
                        S::split8(re, pr_);
                        const uint32_t or_ = mn_off(row2 & 127, g);
#pragma unroll
                        for (int k = 0; k < PARTS; ++k) *reinterpret_cast<uint4*>(blk + k * C::A2_PART + or_) = pr_[k];
                    }
                    if (C::KH == 1 || h == 1) {
                        uint4 pi_[PARTS];
                        S::split8(im, pi_);
                        const uint32_t oi_ = mn_off(row2 & 127, (C::KH == 1 ? Q : 0) + g);
#pragma unroll
                        for (int k = 0; k < PARTS; ++k) *reinterpret_cast<uint4*>(blk + k * C::A2_PART + oi_) = pi_[k];
                    }
                }
            }
            fence_async_smem();
            fence_before();
            __syncthreads();
            fence_after();
            // pass 2 on the tensor cores, one MMA chain per 128-row block: K slices
            // [h KS, h KS + KS) of the complex Q-point DFT, this half's A2 at slice 0
            constexpr int KS = C::K2 / 16 / C::KH;
            if (tid == 0) {
#pragma unroll
                for (int b = 0; b < MB; ++b) {
#pragma unroll
                    for (int kk = 0; kk < KS; ++kk) {
                        const int ks = h * KS + kk;
#pragma unroll
                        for (int pr = 0; pr < NPROD; ++pr) {
                            const uint64_t ad =
                                sdesc(sa + b * C::A2_BLOCK + PA[pr] * C::A2_PART + kk * 4096, 1024, 2048);
                            const uint64_t bd =
                                sdesc(sb2 + PB[pr] * C::B2_PART + (ks >> 2) * C::B2_PANEL + (ks & 3) * 32, 16, 1024);
                            mma_f16(d2 + b * C::NO2, ad, bd, ID2, (ks > 0 || pr > 0) ? 1u : 0u);
                        }
                    }
                }
                mma_commit(&mbar[1]);
            }
            if (!mbar_wait(&mbar[1], phase1)) {
                if (lane == 0) atomicExch(abort_flag, 1);
            }
            phase1 ^= 1u;
            __syncthreads();
            if (*abort_flag) break;
            fence_after();
        }
        if (*abort_flag) {
            aborted = true;
            break;
        }
        // ---------------- epilogue 2: thread = (frame, k1) of each block holds X[k1 + P k2]
#pragma unroll 1
        for (int b = 0; b < MB; ++b) {
            const int row2 = b * 128 + tid, lf = row2 / P, k1 = row2 % P;
            const uint64_t f = f0 + lf;
            const bool act = f < a.frames;
            const float back = fscale[lf] * (float)P;  // undo both scalings (powers of two)
#pragma unroll 1
            for (int k2b = 0; k2b < Q; k2b += 8) {
                float t[16];
                tmem_ld16(d2 + b * C::NO2 + lane_base + 2 * k2b, t);
                if (!act) continue;
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int k = k1 + P * (k2b + q);
                    const float xr = t[2 * q] * back, xi = t[2 * q + 1] * back;
                    if constexpr (OUTK == OUT_HALF) {
                        float2* o2 = reinterpret_cast<float2*>(a.out);
                        const float2 X = make_float2(xr, xi);
                        if (!a.dense) {
                            const uint64_t flat = f * (uint64_t)N + k;
                            if (flat < a.ohalf) __stcs(o2 + flat, X);
                        } else if (k <= N / 2) {
                            __stcs(o2 + f * (uint64_t)(N / 2 + 1) + k, X);
                        }
                    } else {
                        if (k > N / 2) continue;
                        const float p = (OUTK == OUT_POWER_SERIAL) ? fabsf(xr) * 1.41421356237309505f
                                                                   : sqrtf(xr * xr + xi * xi);
                        if (!a.dense) {
                            float* rowp = a.out + f * (uint64_t)N;
                            __stcs(rowp + k, p);
                            if (k != 0 && k != N / 2) __stcs(rowp + (N - k), p);
                        } else {
                            __stcs(a.out + f * (uint64_t)(N / 2 + 1) + k, p);
                        }
                    }
                }
            }
        }
        fence_before();
        __syncthreads();
        fence_after();
        phase ^= 1u;
    }
    // ---------------- release tensor memory (every exit path)
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(C::TMEM_COLS));
    }
    if (aborted && tid == 0) *reinterpret_cast<volatile int*>(err) = 1;
}

template <int P, int Q, int OUTK, int PM>
cudaError_t launch_tcg_t(const FusedArgs& a, int* err, int sms, cudaStream_t st)
{
    using C = TcgCfg<P, Q, PM>;
    if constexpr (!C::FITS) {
        return cudaErrorInvalidValue;
    } else {
        auto k = stft_tcg_kernel<P, Q, OUTK, PM>;
        cudaError_t e = ensure_smem_attr<stft_tcg_kernel<P, Q, OUTK, PM>>(C::SMEM);
        if (e != cudaSuccess) return e;
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, 128, C::SMEM);
        if (e != cudaSuccess) return e;
        // CTAs resident on one SM must also fit its 512 tensor-memory columns
        const int by_tmem = 512 / (int)C::TMEM_COLS;
        const int per_sm = occ < 1 ? 1 : (occ < by_tmem ? occ : by_tmem);
        const uint64_t ntiles = (a.frames + C::FPT - 1) / C::FPT;
        const uint64_t cap = (uint64_t)sms * per_sm;
        const uint64_t grid = ntiles < cap ? ntiles : cap;
        k<<<(unsigned)(grid ? grid : 1), 128, C::SMEM, st>>>(a, err);
        return cudaGetLastError();
    }
}

template <int P, int Q, int PM>
cudaError_t launch_tcg_o(int outk, const FusedArgs& a, int* err, int sms, cudaStream_t st)
{
    if (outk == OUT_HALF) return launch_tcg_t<P, Q, OUT_HALF, PM>(a, err, sms, st);
    if (outk == OUT_POWER_SERIAL) return launch_tcg_t<P, Q, OUT_POWER_SERIAL, PM>(a, err, sms, st);
    return launch_tcg_t<P, Q, OUT_POWER, PM>(a, err, sms, st);
}

template <int P, int Q>
cudaError_t launch_tcg_p(int pm, int outk, const FusedArgs& a, int* err, int sms, cudaStream_t st)
{
    if (pm == PM_BF16X2) return launch_tcg_o<P, Q, PM_BF16X2>(outk, a, err, sms, st);
    if (pm == PM_BF16X3) return launch_tcg_o<P, Q, PM_BF16X3>(outk, a, err, sms, st);
    return launch_tcg_o<P, Q, PM_FP16X2>(outk, a, err, sms, st);
}

template <int R, int PM>
const unsigned char* tc_tables(cudaError_t* e)
{
    // built once per device (the image is a __device__ array, one per
    // device); a failed build (say, attempted while another stream was
    // capturing a graph) is retried by the next call instead of being remembered
    static std::mutex mu;
    static unsigned char* img[64] = {};
    int dev = 0;
    cudaError_t rd = cudaGetDevice(&dev);
    if (rd != cudaSuccess || dev < 0 || dev >= 64) {
        *e = rd != cudaSuccess ? rd : cudaErrorInvalidDevice;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(mu);
    if (img[dev]) {
        *e = cudaSuccess;
        return img[dev];
    }
    void* p = nullptr;
    cudaError_t r;
    if constexpr (R == 16 && PM == 1) r = cudaGetSymbolAddress(&p, g_tc_tab16_1);
    else if constexpr (R == 16 && PM == 2) r = cudaGetSymbolAddress(&p, g_tc_tab16_2);
    else if constexpr (R == 16) r = cudaGetSymbolAddress(&p, g_tc_tab16_3);
    else if constexpr (PM == 1) r = cudaGetSymbolAddress(&p, g_tc_tab32_1);
    else if constexpr (PM == 2) r = cudaGetSymbolAddress(&p, g_tc_tab32_2);
    else r = cudaGetSymbolAddress(&p, g_tc_tab32_3);
    if (r == cudaSuccess) {
        // a private stream: the caller's may be capturing a graph
        cudaStream_t s2 = nullptr;
        r = cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking);
        if (r == cudaSuccess) {
            build_tc_tables_kernel<R, PM><<<8, 256, 0, s2>>>(static_cast<unsigned char*>(p));
            r = cudaGetLastError();
            if (r == cudaSuccess) r = cudaStreamSynchronize(s2);
            cudaStreamDestroy(s2);
        }
    }
    *e = r;
    if (r != cudaSuccess) return nullptr;
    img[dev] = static_cast<unsigned char*>(p);
    return img[dev];
}

template <int R, int OUTK, int PM>
cudaError_t launch_tc2_t(const FusedArgs& a, int* err, int test_stall, int sms, cudaStream_t st)
{
    using C = Tc2Cfg<R, PM>;
    cudaError_t e = cudaSuccess;
    const unsigned char* tab = tc_tables<R, PM>(&e);
    if (e != cudaSuccess) return e;
    auto k = stft_tc2_kernel<R, OUTK, PM>;
    e = ensure_smem_attr<stft_tc2_kernel<R, OUTK, PM>>(C::SMEM);
    if (e != cudaSuccess) return e;
    // one CTA per SM: its tensor memory (TMEM_COLS) and shared memory
    const uint64_t ntiles = (a.frames + C::FPT - 1) / C::FPT;
    const uint64_t grid = ntiles < (uint64_t)sms ? ntiles : (uint64_t)sms;
    k<<<(unsigned)(grid ? grid : 1), kTc2Threads, C::SMEM, st>>>(a, tab, err, test_stall);
    return cudaGetLastError();
}

template <int R, int PM>
cudaError_t launch_tc2_o(int outk, const FusedArgs& a, int* err, int test_stall, int sms, cudaStream_t st)
{
    if (outk == OUT_HALF) return launch_tc2_t<R, OUT_HALF, PM>(a, err, test_stall, sms, st);
    if (outk == OUT_POWER_SERIAL) return launch_tc2_t<R, OUT_POWER_SERIAL, PM>(a, err, test_stall, sms, st);
    return launch_tc2_t<R, OUT_POWER, PM>(a, err, test_stall, sms, st);
}

template <int R>
cudaError_t launch_tc2_p(int pm, int outk, const FusedArgs& a, int* err, int test_stall, int sms, cudaStream_t st)
{
    if (pm == PM_BF16X2) return launch_tc2_o<R, PM_BF16X2>(outk, a, err, test_stall, sms, st);
    if (pm == PM_BF16X3) return launch_tc2_o<R, PM_BF16X3>(outk, a, err, test_stall, sms, st);
    return launch_tc2_o<R, PM_FP16X2>(outk, a, err, test_stall, sms, st);
}

template <int R, int OUTK>
cudaError_t launch_tc_t(const FusedArgs& a, int* err, int sms, cudaStream_t st)
{
    using C = TcCfg<R>;
    auto k = stft_tc_kernel<R, OUTK>;
    const cudaError_t e = ensure_smem_attr<stft_tc_kernel<R, OUTK>>(C::SMEM);
    if (e != cudaSuccess) return e;
    const uint64_t ntiles = (a.frames + C::FPT - 1) / C::FPT;
    // at most two CTAs per SM hold tensor memory at a time (2 x TMEM_COLS <= 512)
    const uint64_t grid = ntiles < (uint64_t)sms * 2 ? ntiles : (uint64_t)sms * 2;
    k<<<(unsigned)(grid ? grid : 1), 128, C::SMEM, st>>>(a, err);
    return cudaGetLastError();
}

}  // namespace

bool tc_supports(int exp) { return exp >= 8 && exp <= 12; }

bool tc_mode_supported(int exp, int pm)
{
    (void)pm;  // every split mode at every size (bf16 hi/mid/lo at 4096 takes pass 2 in K halves)
    return tc_supports(exp);
}

// whether every split mode is available for this frame advance: the
// pipelined forms (windows 2^8 and 2^10) stage a span sized for hop <= N;
// the generic form (2^9, 2^11, 2^12) takes any advance
bool tc_piped(int exp, uint64_t hop) { return (exp != 8 && exp != 10) || hop <= (1ull << exp); }

cudaError_t tc_prepare(int exp, int pm)
{
    cudaError_t e = cudaSuccess;
    if (exp == 8) {
        if (pm == PM_BF16X2) tc_tables<16, PM_BF16X2>(&e);
        else if (pm == PM_BF16X3) tc_tables<16, PM_BF16X3>(&e);
        else tc_tables<16, PM_FP16X2>(&e);
    } else if (exp == 10) {
        if (pm == PM_BF16X2) tc_tables<32, PM_BF16X2>(&e);
        else if (pm == PM_BF16X3) tc_tables<32, PM_BF16X3>(&e);
        else tc_tables<32, PM_FP16X2>(&e);
    }
    return e;  // the generic form (2^9, 2^11, 2^12) builds its tables in each CTA
}

cudaError_t launch_tc(int exp, int outk, int pm, const FusedArgs& a, int* err, int test_stall, int sms,
                      cudaStream_t st)
{
    // the pipelined form stages one tile's input span, sized for hop <= N;
    // the first form (fp16 split only) takes longer frame advances
    const bool piped = tc_piped(exp, a.hop) && (reinterpret_cast<uintptr_t>(a.x) & 3u) == 0;
    if (piped && exp == 8) return launch_tc2_p<16>(pm, outk, a, err, test_stall, sms, st);
    if (piped && exp == 10) return launch_tc2_p<32>(pm, outk, a, err, test_stall, sms, st);
    if (exp == 9) return launch_tcg_p<32, 16>(pm, outk, a, err, sms, st);
    if (exp == 11) return launch_tcg_p<64, 32>(pm, outk, a, err, sms, st);
    if (exp == 12) return launch_tcg_p<64, 64>(pm, outk, a, err, sms, st);
    if (pm != PM_FP16X2) return cudaErrorInvalidValue;
    if (exp == 8) {
        if (outk == OUT_HALF) return launch_tc_t<16, OUT_HALF>(a, err, sms, st);
        if (outk == OUT_POWER_SERIAL) return launch_tc_t<16, OUT_POWER_SERIAL>(a, err, sms, st);
        return launch_tc_t<16, OUT_POWER>(a, err, sms, st);
    }
    if (exp == 10) {
        if (outk == OUT_HALF) return launch_tc_t<32, OUT_HALF>(a, err, sms, st);
        if (outk == OUT_POWER_SERIAL) return launch_tc_t<32, OUT_POWER_SERIAL>(a, err, sms, st);
        return launch_tc_t<32, OUT_POWER>(a, err, sms, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace ocs
