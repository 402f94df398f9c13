// STFT for windows 2^16 .. 2^30 (sm_103a): a four-step FFT in two launches
// up to 2^22, three above.
//
// One frame of N real samples is the M = N/2 point complex FFT of
// z[m] = y[2m] + i y[2m+1] plus the real-input untangle, as in the fused
// kernels; here M = M1 * M2 does not fit one CTA, so with m = c + M2 m1 and
// k = k1 + M1 k2:
//   column pass  Y[k1][c]  = W_M^{c k1} * sum_{m1} z[c + M2 m1] W_{M1}^{m1 k1}
//   row pass     Z[k1 + M1 k2] = sum_c Y[k1][c] W_{M2}^{c k2}
// followed by X[k] = (Z[k] + conj Z[M-k]) + W_N^k (Z[k] - conj Z[M-k]) / i and
// X[k + M] = (Z[k] + conj Z[M-k]) - W_N^k (...) (the window table carries the
// untangle's factor 1/2).
//
// Column pass: a CTA owns 16 (windows 2^16, 2^17) or 8 consecutive columns
// of one frame.  It reads the frame's samples row by row (128 or 64
// contiguous bytes per row), applies the
// window, runs 8 M1-point FFTs with the fused kernels' Stockham core, applies
// W_M^{c k1} and writes Y row-major to a scratch area (again 64-byte rows).
// Row pass: a CTA owns 8 rows k1 and their 8 mirror rows M1 - k1 (row M1/2
// stands in for the mirror of row 0), so every Z[M-k] it needs is its own.
// It runs 16 M2-point FFTs, then writes outputs with lanes over k1, i.e. 8
// consecutive bins per (k2) run.
//
// Above 2^22 the column FFT would exceed a CTA, so M = P1 * P2 * Q and the
// column length P = P1 * P2 splits once more (m = c + Q (a + P2 m1),
// k1 = k1a + P1 k1b):
//   column pass  U[k1a][c + Q a] = W_P^{a k1a} sum_{m1} z[c + Q a + Q P2 m1] W_{P1}^{m1 k1a}
//   middle pass  Y[k1a + P1 k1b][c] = W_M^{c k1} sum_a U[k1a][c + Q a] W_{P2}^{a k1b}
//   row pass     as above, over P rows of Q points.
// The column pass is the two-launch column pass with Q P2 columns and the
// twiddle exponent taken from the column's block (c + Q a) & ~(Q - 1) = Q a,
// since W_P^{a k1a} = W_M^{Q a k1a}.
//
// DC removal subtracts the mean of the windowed frame; in the transform that
// changes bin 0 only (to zero), which is what the row pass writes.  The
// reference's EXPC runs any exponent >= 12 through a radix-2 Stockham
// (RunnerCommon.cpp:278-289, Serial/src/functionImpl.cpp:186-270).
#include "stft_fused_kernel.cuh"

namespace ocs {
namespace {

constexpr int kTileC = 8;  // columns per middle-pass CTA (column pass: large_col_tile)
constexpr int kTileR = 8;  // rows (and as many mirror rows) per row-pass CTA

// Column-pass buffer stride: = 2 (mod 8) float2.  An 8-byte shared access is
// served per half-warp; in the staging loops a half-warp is 4 rows x 4 lanes,
// lane q on columns 2q and 2q+1, so the columns must start 4 bank pairs
// apart for the 16 lanes to hit 16 distinct ones (with = 4 (mod 8) lanes q
// and q + 2 collided: 2.9 wavefronts per load where 2 are needed).
__host__ __device__ constexpr int large_col_stride(int exp1)
{
    return fused_buf_stride(exp1) + ((2 - fused_buf_stride(exp1) % 8) + 8) % 8;
}
// Row-pass buffers: row r starts at r * large_row_stride + large_row_shift(r),
// the stride a multiple of 16 float2 and the shift 0, 8, 4, 12, 2, 10, 6, 14
// for r mod 8.  The four rows a warp transforms at window 2^8 (8 lanes per row
// on 8 consecutive slots) then tile the 16 bank pairs twice, and so do the
// output loop's reads of 8 rows at 4 consecutive columns.
__host__ __device__ constexpr int large_row_stride(int exp2) { return (fused_buf_stride(exp2) + 14 + 15) / 16 * 16; }
__device__ __forceinline__ int large_row_shift(int r) { return 8 * (r & 1) + 4 * ((r >> 1) & 1) + 2 * ((r >> 2) & 1); }

__host__ __device__ constexpr int large_l1(int exp) { return exp / 2; }         // log2 M1
__host__ __device__ constexpr int large_l2(int exp) { return exp - 1 - exp / 2; }  // log2 M2

// exp(-2 pi i j / L) from a two-level table: lo[j & 1023] * hi[j >> 10]
__device__ __forceinline__ float2 tw2l(const float2* lo, const float2* hi, uint64_t j)
{
    return cmul(lo[j & 1023u], hi[j >> 10]);
}

// ---------------------------------------------------------------- column pass
// Column FFTs of up to 512 points (windows 2^16 .. 2^19) keep the CTA's
// window coefficients in registers and take 4 consecutive frames of the same
// columns per CTA; the larger ones (more chunks per thread, or 1024 threads
// at 64 registers) take one frame per CTA and read the window each time.
//
// A CTA owns 16 columns (rows of 128 bytes, 8 lanes per row) where that keeps
// it at 256 threads (column FFTs of 256 points, windows 2^16 and 2^17), else
// 8: each warp-wide row load then touches half as many cache lines.
__host__ __device__ constexpr int large_col_tile(int exp1)
{
    return 16 * (fused_M(exp1) / fused_cfg(exp1).R) <= 256 ? 16 : 8;
}
// Its buffer stride: with 16 columns an odd number of float2, so that a
// half-warp's 8-byte staging accesses (2 rows x 8 lanes, lane q on columns 2q
// and 2q + 1) land on 16 distinct bank pairs; with 8 columns the stride of
// the middle pass.
__host__ __device__ constexpr int large_col_stride_t(int exp1, int tc)
{
    return tc == 16 ? (fused_buf_stride(exp1) | 1) : large_col_stride(exp1);
}
__host__ __device__ constexpr bool large_col_cache_win(int exp1)
{
    return fused_M(exp1) / (2 * (fused_M(exp1) / fused_cfg(exp1).R)) <= 8 &&
           large_col_tile(exp1) * (fused_M(exp1) / fused_cfg(exp1).R) <= 256;
}
__host__ __device__ constexpr int large_col_frames(int exp1) { return large_col_cache_win(exp1) ? 4 : 1; }

// four window coefficients at real index i (a multiple of 4); no table: 1/2
__device__ __forceinline__ float4 large_win4(const float* win, uint32_t i)
{
    return win ? *reinterpret_cast<const float4*>(win + i) : make_float4(0.5f, 0.5f, 0.5f, 0.5f);
}

template <int EXP1>
__global__ void __launch_bounds__(large_col_tile(EXP1) * (fused_M(EXP1) / fused_cfg(EXP1).R))
    large_columns_kernel(const LargeArgs a)
{
    using K = Core<EXP1>;
    constexpr int M1 = K::M, R = K::R, T = K::T;
    constexpr int TC = large_col_tile(EXP1);  // columns
    constexpr int QR = TC / 2;                // float4 chunks per row
    constexpr int NT = TC * T;                // threads
    constexpr int NE = M1 * QR / NT;          // float4 row chunks per thread (= R / 2)
    constexpr int BS = large_col_stride_t(EXP1, TC);
    extern __shared__ float2 sbuf[];  // TC column buffers of BS slots
    const int tid = threadIdx.x;
    const uint64_t M2 = a.m2;
    const uint64_t tiles = M2 / TC;
    const uint64_t fg = blockIdx.x / tiles;  // group of FPC frames within this launch
    const uint64_t c0 = (blockIdx.x % tiles) * TC;
    const uint64_t N = 2 * (uint64_t)M1 * M2;
    const bool aligned = (a.hop & 3) == 0 && (reinterpret_cast<uintptr_t>(a.x) & 15) == 0;
    // this CTA's window coefficients: chunk j is row m1 = e / QR, columns 2q,
    // 2q+1 (q = e % QR) with e = tid + j NT; row m1 starts at real index
    // 2 (c0 + M2 m1), a multiple of 16
    constexpr bool CACHE_WIN = large_col_cache_win(EXP1);
    constexpr int FPC = large_col_frames(EXP1);
    float4 wv[CACHE_WIN ? NE : 1];
    if constexpr (CACHE_WIN) {
#pragma unroll
        for (int j = 0; j < NE; ++j) {
            const int e = tid + j * NT, m1 = e / QR, q = e % QR;
            wv[j] = large_win4(a.win, 2u * ((uint32_t)c0 + (uint32_t)M2 * (uint32_t)m1) + 4u * (uint32_t)q);
        }
    }
    const int col = tid / T, t = tid % T;
    float2* buf = sbuf + col * BS;
    const uint64_t c = c0 + col;

#pragma unroll 1
    for (int ff = 0; ff < FPC; ++ff) {
        const uint64_t fl = fg * FPC + ff;  // frame within this launch
        if (fl >= a.frames_launch) break;
        const uint64_t f = a.f0 + fl;
        const uint64_t s0 = f * a.hop;
        if (ff > 0) __syncthreads();  // the previous frame's reads of the buffers are over
        // rows of TC complex samples (64 or 128 bytes)
        if (aligned && f < a.frames_total && s0 + N <= a.n) {
            // frame inside the signal and 16-byte aligned: QR threads per
            // row, a float4 (two complex samples) each
            const float* xf = a.x + s0;
            auto chunk = [&](int e, const float4& w) {
                const int m1 = e / QR, q = e % QR;
                const uint32_t i = 2u * ((uint32_t)c0 + (uint32_t)M2 * (uint32_t)m1) + 4u * (uint32_t)q;
                const float4 xv = *reinterpret_cast<const float4*>(xf + i);
                sbuf[(2 * q) * BS + K::pd(m1)] = make_float2(xv.x * w.x, xv.y * w.y);
                sbuf[(2 * q + 1) * BS + K::pd(m1)] = make_float2(xv.z * w.z, xv.w * w.w);
            };
            if constexpr (CACHE_WIN) {
#pragma unroll
                for (int j = 0; j < NE; ++j) chunk(tid + j * NT, wv[j]);
            } else {
                for (int e = tid; e < M1 * QR; e += NT) {
                    const uint32_t i = 2u * ((uint32_t)c0 + (uint32_t)M2 * (uint32_t)(e / QR)) + 4u * (uint32_t)(e % QR);
                    chunk(e, large_win4(a.win, i));
                }
            }
        } else {
            // lane pairs take one row, samples past the signal end read as zero
            for (int e = tid; e < M1 * TC; e += NT) {
                const int cc = e % TC, m1 = e / TC;
                const uint64_t m = c0 + cc + M2 * (uint64_t)m1;  // complex index in the frame
                const uint64_t i = 2 * m;                         // real sample index in the frame
                const uint64_t g = s0 + i;
                float xr = 0.0f, xi = 0.0f;
                if (f < a.frames_total) {
                    if (g < a.n) xr = a.x[g];
                    if (g + 1 < a.n) xi = a.x[g + 1];
                }
                const float2 w = a.win ? *reinterpret_cast<const float2*>(a.win + i) : make_float2(0.5f, 0.5f);
                sbuf[cc * BS + K::pd(m1)] = make_float2(xr * w.x, xi * w.y);
            }
        }
        __syncthreads();
        float2 v[R];
#pragma unroll
        for (int u = 0; u < R; ++u) v[u] = buf[K::pd(t + u * T)];
        K::fft(v, buf, a.tw1, t);  // slot u holds column FFT bin k1 = t + u*T
        __syncthreads();
        // W_M^{c k1}, k1 = t + u T: a two-level lookup at u = 0 and 8, then
        // products with W_M^{c T} (at most 7 rounding steps)
        const uint64_t ce = c & a.col_mask;  // c, or the block Q a of the three-pass form
        const float2 step = tw2l(a.twm_lo, a.twm_hi, ce * (uint64_t)T);
        float2 w = make_float2(1.0f, 0.0f);
#pragma unroll
        for (int u = 0; u < R; ++u) {
            const int k1 = t + u * T;
            w = (u % 8 == 0) ? tw2l(a.twm_lo, a.twm_hi, ce * (uint64_t)k1) : cmul(w, step);
            buf[K::pd(k1)] = cmul(v[u], w);
        }
        __syncthreads();
        // Y row-major: row k1 holds this CTA's TC columns at c0 (64 or 128
        // bytes), written as QR float4 (two complex values) per row
        float2* y = a.scratch + fl * (uint64_t)M1 * M2;
        for (int e = tid; e < M1 * QR; e += NT) {
            const int k1 = e / QR, q = e % QR;
            const float2 lo = sbuf[(2 * q) * BS + K::pd(k1)], hi = sbuf[(2 * q + 1) * BS + K::pd(k1)];
            *reinterpret_cast<float4*>(y + (uint64_t)k1 * M2 + c0 + 2 * q) = make_float4(lo.x, lo.y, hi.x, hi.y);
        }
    }
}

// ---------------------------------------------------------------- middle pass
// Three-pass form: a CTA owns 8 consecutive columns c of block k1a of one
// frame.  It reads rows a (P2 of them, 8 complex values = 64 bytes each, at
// U + k1a Q P2 + Q a + c0), runs 8 P2-point FFTs on the Stockham core,
// multiplies W_M^{c (k1a + P1 k1b)} and writes rows k1a + P1 k1b of Y.
// Per launch: m1 = P1, m2 = Q, scratch = U, scratch2 = Y.
template <int EXPM>
__global__ void __launch_bounds__(kTileC * (fused_M(EXPM) / fused_cfg(EXPM).R))
    large_middle_kernel(const LargeArgs a)
{
    using K = Core<EXPM>;
    constexpr int P2 = K::M, R = K::R, T = K::T;
    constexpr int NT = kTileC * T;
    constexpr int BS = large_col_stride(EXPM);
    extern __shared__ float2 sbuf[];
    const int tid = threadIdx.x;
    const uint64_t P1 = a.m1, Q = a.m2;
    const uint64_t M = P1 * (uint64_t)P2 * Q;
    const uint64_t ctiles = Q / kTileC;
    const uint64_t c0 = (blockIdx.x % ctiles) * kTileC;
    const uint64_t k1a = (blockIdx.x / ctiles) % P1;
    const uint64_t fl = blockIdx.x / (ctiles * P1);
    const float2* u = a.scratch + fl * M + k1a * (Q * P2);
    for (int e = tid; e < P2 * 4; e += NT) {
        const int r = e >> 2, q = e & 3;
        const float4 d = *reinterpret_cast<const float4*>(u + (uint64_t)r * Q + c0 + 2 * q);
        sbuf[(2 * q) * BS + K::pd(r)] = make_float2(d.x, d.y);
        sbuf[(2 * q + 1) * BS + K::pd(r)] = make_float2(d.z, d.w);
    }
    __syncthreads();
    const int col = tid / T, t = tid % T;
    float2* buf = sbuf + col * BS;
    const uint64_t c = c0 + col;
    float2 v[R];
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = buf[K::pd(t + i * T)];
    K::fft(v, buf, a.tw3, t);  // slot i: output k1b = t + i T
    __syncthreads();
    // W_M^{c (k1a + P1 k1b)}: a two-level lookup at i = 0 and 8, products with
    // W_M^{c P1 T} between (exponents below M: c < Q, k1a + P1 k1b < P1 P2)
    const float2 step = tw2l(a.twm_lo, a.twm_hi, c * P1 * (uint64_t)T);
    float2 w = make_float2(1.0f, 0.0f);
#pragma unroll
    for (int i = 0; i < R; ++i) {
        const int k1b = t + i * T;
        w = (i % 8 == 0) ? tw2l(a.twm_lo, a.twm_hi, c * (k1a + P1 * (uint64_t)k1b)) : cmul(w, step);
        buf[K::pd(k1b)] = cmul(v[i], w);
    }
    __syncthreads();
    float2* y = a.scratch2 + fl * M;
    for (int e = tid; e < P2 * 4; e += NT) {
        const int kb = e >> 2, q = e & 3;
        const float2 lo = sbuf[(2 * q) * BS + K::pd(kb)], hi = sbuf[(2 * q + 1) * BS + K::pd(kb)];
        *reinterpret_cast<float4*>(y + (k1a + P1 * (uint64_t)kb) * Q + c0 + 2 * q) = make_float4(lo.x, lo.y, hi.x, hi.y);
    }
}

// ---------------------------------------------------------------- row pass
template <int EXP2, int OUTK>
__global__ void __launch_bounds__(2 * kTileR * (fused_M(EXP2) / fused_cfg(EXP2).R))
    large_rows_kernel(const LargeArgs a)
{
    using K = Core<EXP2>;
    constexpr int M2 = K::M, R = K::R, T = K::T;
    constexpr int BS = large_row_stride(EXP2);
    extern __shared__ float2 sbuf[];  // 2*kTileR row buffers (large_row_stride / large_row_shift)
    const int tid = threadIdx.x;
    const uint64_t M1 = a.m1;
    const uint64_t M = M1 * M2;
    const uint64_t N = 2 * M;
    const uint64_t blocks = M1 / (2 * kTileR);
    const uint64_t fl = blockIdx.x / blocks;
    const uint64_t b = blockIdx.x % blocks;
    const uint64_t f = a.f0 + fl;

    // slot s < kTileR: row b*8 + s; slot kTileR + s: its mirror M1 - row,
    // except that row 0's mirror slot holds row M1/2
    auto row_of = [&](int s) -> uint64_t {
        const uint64_t d = b * kTileR + (uint64_t)(s % kTileR);
        if (s < kTileR) return d;
        return d == 0 ? M1 / 2 : M1 - d;
    };
    const int rs = tid / T, t = tid % T;
    const float2* y = a.scratch + fl * M;
    float2* buf = sbuf + rs * BS + large_row_shift(rs);
    {
        const float2* yr = y + row_of(rs) * M2;
        float2 v[R];
#pragma unroll
        for (int u = 0; u < R; ++u) v[u] = yr[t + u * T];
        K::fft(v, buf, a.tw2, t);  // slot u: Z[k1 + M1 (t + u T)]
        __syncthreads();
#pragma unroll
        for (int u = 0; u < R; ++u) buf[K::pd(t + u * T)] = v[u];
    }
    __syncthreads();
    if (f >= a.frames_total) return;

    // outputs: lanes over the 8 rows of a slot group, then over k2.  Thread
    // tid keeps slot (tid & 7) of each group (first the rows, then their
    // mirrors) and steps k2 by 16, so everything that depends on the slot is
    // formed once per group.
    const bool dc = a.remove_dc != 0;
    const uint32_t m1 = (uint32_t)M1, m2 = (uint32_t)M2;
    if constexpr (OUTK == OUT_POWER || OUTK == OUT_POWER_SERIAL) {
        // Power: one untangle at k gives X[k] and X[M + k], and for a real
        // frame |X[N - k]| = |X[k]|, |X[M - k]| = |X[M + k]|, so only the 8
        // rows are untangled and their mirrors (which hold the partners)
        // come for free.  Row 0 pairs with itself (k2 with M2 - k2) and so
        // does row M1/2 (k2 with M2 - 1 - k2): the first CTA's slot 0 takes
        // row 0 for k2 < M2/2, row M1/2 for the other half, and k = M/2 last.
        const int s = tid & (kTileR - 1);
        const bool special = b == 0 && s == 0;
        const uint32_t k1 = (uint32_t)row_of(s);
        const float2* zs = sbuf + s * BS + large_row_shift(s);
        const float2* zp = sbuf + (s + kTileR) * BS + large_row_shift(s + kTileR);
        const float2 wk1 = special ? tw2l(a.twn_lo, a.twn_hi, m1 / 2) : tw2l(a.twn_lo, a.twn_hi, k1);
        float* ro = a.out + f * (a.dense ? M + 1 : N);
        auto emit = [&](uint32_t k, float2 A, float2 B, float2 w) {
            float2 ev, wo;
            K::untangle(A, B, w, ev, wo);
            float2 X0 = make_float2(ev.x + wo.x, ev.y + wo.y);        // X[k]
            const float2 X1 = make_float2(ev.x - wo.x, ev.y - wo.y);  // X[k + M]
            if (dc && k == 0) X0 = make_float2(0.0f, 0.0f);
            const float p0 = power_of<OUTK>(X0), p1 = power_of<OUTK>(X1);
            const bool mirror = k != 0 && k != (uint32_t)(M / 2);
            if (!a.dense) {
                __stcs(ro + k, p0);
                __stcs(ro + (k + M), p1);
                if (mirror) {
                    __stcs(ro + (N - k), p0);
                    __stcs(ro + (M - k), p1);
                }
            } else {
                __stcs(ro + k, p0);
                if (mirror) __stcs(ro + (M - k), p1);
                if (k == 0) __stcs(ro + M, p1);
            }
        };
        if (!special) {
#pragma unroll 2
            for (uint32_t k2 = (uint32_t)tid / kTileR; k2 < m2; k2 += blockDim.x / kTileR)
                emit(k1 + m1 * k2, zs[K::pd((int)k2)], zp[K::pd((int)(m2 - 1 - k2))], cmul(wk1, a.tw2[k2]));
        } else {
            for (uint32_t k2 = (uint32_t)tid / kTileR; k2 < m2; k2 += blockDim.x / kTileR) {
                if (k2 < m2 / 2) {
                    emit(m1 * k2, zs[K::pd((int)k2)], zs[K::pd((int)((m2 - k2) & (m2 - 1)))], a.tw2[k2]);
                } else {
                    const uint32_t hk = k2 - m2 / 2;  // row M1/2 sits in slot kTileR
                    emit(m1 / 2 + m1 * hk, zp[K::pd((int)hk)], zp[K::pd((int)(m2 - 1 - hk))], cmul(wk1, a.tw2[hk]));
                }
            }
            if (tid == 0) {
                const float2 A = zs[K::pd((int)(m2 / 2))];
                emit((uint32_t)(M / 2), A, A, a.tw2[m2 / 2]);
            }
        }
    } else {
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
        const int s = (tid & (kTileR - 1)) + kTileR * h;
        const uint32_t k1 = (uint32_t)row_of(s);
        // partner Z[M - k]: row (M1 - k1) mod M1; column M2-1-k2, or (M2-k2) mod M2 for row 0
        const int ps = (k1 == 0 || k1 == m1 / 2) ? s : (s < kTileR ? s + kTileR : s - kTileR);
        const bool row0 = k1 == 0;
        const float2* zs = sbuf + s * BS + large_row_shift(s);
        const float2* zp = sbuf + ps * BS + large_row_shift(ps);
        // W_N^k for k = k1 + M1 k2: W_N^{k1} W_{2 M2}^{k2}; the second factor
        // is the untangle table of the M2-point plan (its first M2 entries)
        const float2 wk1 = tw2l(a.twn_lo, a.twn_hi, k1);
        float* ro = a.out + f * N;
        float* rod = a.out + f * (M + 1);
        float2* o2 = reinterpret_cast<float2*>(a.out);
#pragma unroll 2
        for (uint32_t k2 = (uint32_t)tid / kTileR; k2 < m2; k2 += blockDim.x / kTileR) {
            const uint32_t pk2 = row0 ? ((m2 - k2) & (m2 - 1)) : (m2 - 1 - k2);
            const float2 A = zs[K::pd((int)k2)];
            const float2 B = zp[K::pd((int)pk2)];
            const uint32_t k = k1 + m1 * k2;
            float2 ev, wo;
            K::untangle(A, B, cmul(wk1, a.tw2[k2]), ev, wo);
            float2 X0 = make_float2(ev.x + wo.x, ev.y + wo.y);        // X[k]
            const float2 X1 = make_float2(ev.x - wo.x, ev.y - wo.y);  // X[k + M]
            if (dc && k == 0) X0 = make_float2(0.0f, 0.0f);
            if constexpr (OUTK == OUT_PLANES) {
                a.out[f * N + k] = X0.x;
                a.out_im[f * N + k] = X0.y;
                a.out[f * N + k + M] = X1.x;
                a.out_im[f * N + k + M] = X1.y;
            } else if constexpr (OUTK == OUT_HALF) {
                if (!a.dense) {
                    const uint64_t flat = f * N + k;
                    if (flat < a.ohalf) __stcs(o2 + flat, X0);
                    if (flat + M < a.ohalf) __stcs(o2 + flat + M, X1);
                } else {
                    float2* rc = o2 + f * (M + 1);
                    __stcs(rc + k, X0);
                    if (k == 0) __stcs(rc + M, X1);
                }
            } else {
                const float p0 = power_of<OUTK>(X0), p1 = power_of<OUTK>(X1);
                if (!a.dense) {
                    __stcs(ro + k, p0);
                    __stcs(ro + k + M, p1);
                } else {
                    __stcs(rod + k, p0);
                    if (k == 0) __stcs(rod + M, p1);
                }
            }
        }
    }
    }
}

__global__ void build_two_level_kernel(float2* lo, float2* hi, uint64_t L, uint64_t nhi)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < 1024 + nhi;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t j = i < 1024 ? i : (i - 1024) * 1024;
        double s, c;
        sincospi(-2.0 * (double)(j % L) / (double)L, &s, &c);
        const float2 w = make_float2((float)c, (float)s);
        if (i < 1024) lo[i] = w;
        else hi[i - 1024] = w;
    }
}

template <int EXP1>
cudaError_t launch_columns_t(const LargeArgs& a, uint64_t frames, cudaStream_t st)
{
    constexpr int T = fused_M(EXP1) / fused_cfg(EXP1).R;
    constexpr int TC = large_col_tile(EXP1);
    constexpr size_t smem = (size_t)TC * large_col_stride_t(EXP1, TC) * sizeof(float2);
    auto k = large_columns_kernel<EXP1>;
    const cudaError_t e = ensure_smem_attr<large_columns_kernel<EXP1>>(smem);
    if (e != cudaSuccess) return e;
    constexpr int FPC = large_col_frames(EXP1);
    const uint64_t grid = (frames + FPC - 1) / FPC * (a.m2 / TC);
    LargeArgs b = a;
    b.frames_launch = frames;
    k<<<(unsigned)grid, TC * T, smem, st>>>(b);
    return cudaGetLastError();
}

template <int EXP2, int OUTK>
cudaError_t launch_rows_t(const LargeArgs& a, uint64_t frames, cudaStream_t st)
{
    constexpr int T = fused_M(EXP2) / fused_cfg(EXP2).R;
    constexpr size_t smem = (size_t)2 * kTileR * large_row_stride(EXP2) * sizeof(float2);
    auto k = large_rows_kernel<EXP2, OUTK>;
    const cudaError_t e = ensure_smem_attr<large_rows_kernel<EXP2, OUTK>>(smem);
    if (e != cudaSuccess) return e;
    const uint64_t grid = frames * (a.m1 / (2 * kTileR));
    k<<<(unsigned)grid, 2 * kTileR * T, smem, st>>>(a);
    return cudaGetLastError();
}

template <int EXP2>
cudaError_t launch_rows_e(int outk, const LargeArgs& a, uint64_t frames, cudaStream_t st)
{
    switch (outk) {
    case OUT_POWER: return launch_rows_t<EXP2, OUT_POWER>(a, frames, st);
    case OUT_POWER_SERIAL: return launch_rows_t<EXP2, OUT_POWER_SERIAL>(a, frames, st);
    case OUT_HALF: return launch_rows_t<EXP2, OUT_HALF>(a, frames, st);
    case OUT_PLANES: return launch_rows_t<EXP2, OUT_PLANES>(a, frames, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int EXPM>
cudaError_t launch_middle_t(const LargeArgs& a, uint64_t frames, cudaStream_t st)
{
    constexpr int T = fused_M(EXPM) / fused_cfg(EXPM).R;
    constexpr size_t smem = (size_t)kTileC * large_col_stride(EXPM) * sizeof(float2);
    const cudaError_t e = ensure_smem_attr<large_middle_kernel<EXPM>>(smem);
    if (e != cudaSuccess) return e;
    const uint64_t grid = frames * a.m1 * (a.m2 / kTileC);
    large_middle_kernel<EXPM><<<(unsigned)grid, kTileC * T, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_columns(int l1, const LargeArgs& a, uint64_t frames, cudaStream_t st)
{
    switch (l1 + 1) {  // EXP1: the column FFT is the core of window 2^EXP1
    case 9: return launch_columns_t<9>(a, frames, st);
    case 10: return launch_columns_t<10>(a, frames, st);
    case 11: return launch_columns_t<11>(a, frames, st);
    case 12: return launch_columns_t<12>(a, frames, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_rows(int l3, int outk, const LargeArgs& a, uint64_t frames, cudaStream_t st)
{
    switch (l3 + 1) {
    case 8: return launch_rows_e<8>(outk, a, frames, st);
    case 9: return launch_rows_e<9>(outk, a, frames, st);
    case 10: return launch_rows_e<10>(outk, a, frames, st);
    case 11: return launch_rows_e<11>(outk, a, frames, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_middle(int l2, const LargeArgs& a, uint64_t frames, cudaStream_t st)
{
    switch (l2 + 1) {
    case 6: return launch_middle_t<6>(a, frames, st);
    case 7: return launch_middle_t<7>(a, frames, st);
    case 8: return launch_middle_t<8>(a, frames, st);
    case 9: return launch_middle_t<9>(a, frames, st);
    case 10: return launch_middle_t<10>(a, frames, st);
    case 11: return launch_middle_t<11>(a, frames, st);
    case 12: return launch_middle_t<12>(a, frames, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool large_supports(int exp) { return exp >= kLargeMinExp && exp <= kLargeMaxExp; }

// Two passes up to 2^22 (column FFT 2^(exp/2), rows of the rest).  Above,
// rows of Q = 2^l3 points (l3 <= 10, the largest row pass), a column FFT of
// 2^l1 (8 <= l1 <= 11) and a middle FFT of 2^l2 (5 <= l2 <= 11), l1 >= l2 as
// close as the ranges allow.
LargePlan large_plan(int exp)
{
    if (exp <= 22) return LargePlan{2, large_l1(exp), 0, large_l2(exp)};
    const int total = exp - 1;
    for (int l3 = 10; l3 >= 7; --l3) {
        const int rest = total - l3;
        const int l1 = (rest + 1) / 2 < 8 ? 8 : ((rest + 1) / 2 > 11 ? 11 : (rest + 1) / 2);
        const int l2 = rest - l1;
        if (l2 >= 5 && l2 <= 11) return LargePlan{3, l1, l2, l3};
    }
    return LargePlan{0, 0, 0, 0};
}

cudaError_t build_two_level(float2* lo, float2* hi, uint64_t L, cudaStream_t st)
{
    const uint64_t nhi = (L + 1023) / 1024;
    build_two_level_kernel<<<64, 256, 0, st>>>(lo, hi, L, nhi);
    return cudaGetLastError();
}

cudaError_t launch_large(int exp, int outk, const LargeArgs& a, uint64_t frames, cudaStream_t st)
{
    if (!large_supports(exp) || frames == 0) return cudaErrorInvalidValue;
    const LargePlan pl = large_plan(exp);
    if (pl.passes == 0) return cudaErrorInvalidValue;
    const uint64_t q = 1ull << pl.l3;
    LargeArgs c = a;  // column pass: FFT of 2^l1, columns = M / 2^l1
    c.m1 = 1ull << pl.l1;
    c.m2 = 1ull << (pl.l2 + pl.l3);
    c.col_mask = pl.passes == 3 ? ~(q - 1) : ~0ull;
    cudaError_t e = launch_columns(pl.l1, c, frames, st);
    if (e != cudaSuccess) return e;
    LargeArgs r = a;  // row pass: rows of Q points, M / Q of them
    r.m1 = 1ull << (pl.l1 + pl.l2);
    r.m2 = q;
    if (pl.passes == 3) {
        LargeArgs m = a;
        m.m1 = 1ull << pl.l1;
        m.m2 = q;
        e = launch_middle(pl.l2, m, frames, st);
        if (e != cudaSuccess) return e;
        r.scratch = a.scratch2;
    }
    return launch_rows(pl.l3, outk, r, frames, st);
}

}  // namespace ocs
