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

#include <cuda_fp16.h>

#include <cstdint>

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
    uint32_t phase = 0;
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
    if (aborted && tid == 0) atomicExch(err, 1);
}

template <int R, int OUTK>
cudaError_t launch_tc_t(const FusedArgs& a, int* err, int sms, cudaStream_t st)
{
    using C = TcCfg<R>;
    auto k = stft_tc_kernel<R, OUTK>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const uint64_t ntiles = (a.frames + C::FPT - 1) / C::FPT;
    // at most two CTAs per SM hold tensor memory at a time (2 x TMEM_COLS <= 512)
    const uint64_t grid = ntiles < (uint64_t)sms * 2 ? ntiles : (uint64_t)sms * 2;
    k<<<(unsigned)(grid ? grid : 1), 128, C::SMEM, st>>>(a, err);
    return cudaGetLastError();
}

}  // namespace

bool tc_supports(int exp) { return exp == 8 || exp == 10; }

cudaError_t launch_tc(int exp, int outk, const FusedArgs& a, int* err, int sms, cudaStream_t st)
{
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
