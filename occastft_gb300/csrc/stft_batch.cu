// Uneven batch in one persistent launch.
//
// Many requests (each its own signal, window exponent 2^6..2^13, overlap,
// window kind and output layout) are cut into tiles of consecutive frames.
// A persistent grid pulls tiles from a device queue with one atomic per tile
// and runs the fused STFT body specialised for the tile's window size; the
// output kind is read per request.  Tiles are ordered by (window, output
// kind) on the host so that concurrently running CTAs mostly share one code
// path.
#include "stft_pair_kernel.cuh"
#include "stft_tpfl_body.cuh"

namespace ocs {

// frames of the next tile a CTA sends toward L2 when it claims that tile
// (-DOCS_BATCH_CLAIM_PREFETCH builds variant libraries for sweeps)
#ifndef OCS_BATCH_CLAIM_PREFETCH
#define OCS_BATCH_CLAIM_PREFETCH 16
#endif
constexpr uint32_t kBatchClaimPrefetch = OCS_BATCH_CLAIM_PREFETCH;

constexpr int kBatchMinExp = 6;
constexpr int kBatchMaxExp = 13;

__host__ __device__ constexpr size_t batch_group_smem(int exp)
{
    return (size_t)fused_fpc(exp) * fused_buf_stride(exp) * 8 + (size_t)(256 / 32) * 4 + 16;
}
// power tiles of windows 2^9, 2^10 and 2^12 run the two-frames-per-FFT body
__host__ __device__ constexpr bool batch_pair_exp(int exp) { return exp == 9 || exp == 10 || exp == 12; }
__host__ __device__ constexpr size_t batch_pair_smem(int exp)
{
    return (size_t)pair_ppc(exp) * pair_buf_stride(exp) * 8 + (size_t)(256 / 32) * 8 + 16;
}
__host__ __device__ constexpr size_t batch_frames_smem()
{
    size_t m = 0;
    for (int e = kBatchMinExp; e <= kBatchMaxExp; ++e) {
        m = batch_group_smem(e) > m ? batch_group_smem(e) : m;
        if (batch_pair_exp(e)) m = batch_pair_smem(e) > m ? batch_pair_smem(e) : m;
    }
    return (m + 15) / 16 * 16;
}
// Twiddle and window tables of windows up to 2^11 are copied into shared
// memory behind the frame buffers (and re-copied only when a tile's plan or
// window table differs from the previous tile's).  2^12 and 2^13 build the
// two-level twiddle table there instead (128 + N/128 entries) and read their
// window through L1: their full tables would take shared memory from L1,
// which the frames' direct loads need (all windows measured slower with the
// 2^12 tables resident).
constexpr int kBatchSmemTabMaxExp = 11;
__host__ __device__ constexpr size_t batch_tab_smem()
{
    size_t m = 0;
    for (int e = kBatchMinExp; e <= kBatchMaxExp; ++e) {
        const size_t b = e <= kBatchSmemTabMaxExp ? (size_t)fused_tw_size(e) * 8 + ((size_t)1 << e) * 4
                                                  : fused_tw2_entries(e) * 8;
        m = b > m ? b : m;
        if (batch_pair_exp(e)) m = pair_tab_bytes(e) > m ? pair_tab_bytes(e) : m;
    }
    return m;
}
__host__ __device__ constexpr size_t batch_smem_ct() { return batch_frames_smem() + batch_tab_smem(); }

template <int EXP>
__device__ __forceinline__ void batch_tile(const FusedArgs& a, uint64_t f0, uint32_t nf, float2* smem,
                                           const float2** s_tw, const float** s_win)
{
    static_assert(fused_cta_threads(EXP) == 256, "batch CTAs have 256 threads");
    if constexpr (EXP == 7 || EXP == 8) {
        // power tiles of 2^7 and 2^8: the lanes-per-frame body (N/64 lanes per
        // frame, the FFT in registers), each warp taking groups of F frames
        // through its own padded rows in the frame region; its twiddle tables
        // and the window (as float4s) behind them.  The reference layout needs
        // a 16-byte-aligned output for its row stores.
        const bool power = a.outk == OUT_POWER || a.outk == OUT_POWER_SERIAL;
        if (power && a.cs != 0 && (a.dense || (reinterpret_cast<uintptr_t>(a.out) & 15u) == 0)) {
            using C = TplCfg<EXP>;
            constexpr int L = C::L, F = C::F, RS = C::RS, N = C::N;
            static_assert((size_t)8 * F * RS * 4 <= batch_frames_smem(), "rows fit the frame region");
            const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
            float2* s_tw1 = reinterpret_cast<float2*>(reinterpret_cast<char*>(smem) + batch_frames_smem());
            float2* s_tw2 = s_tw1 + 32 * L;
            float4* sw4 = reinterpret_cast<float4*>(s_tw2 + 17 * L);
            const float2* marker = reinterpret_cast<const float2*>(&tpl_tab<EXP>());
            const bool new_tw = *s_tw != marker, new_win = *s_win != a.win;
            if (new_tw || new_win) {
                __syncthreads();  // the previous tile's table reads are over
                if (new_tw) tpl_tables<EXP>(s_tw1, s_tw2, tid, 256);
                for (int i = tid; i < N / 4; i += 256) sw4[i] = reinterpret_cast<const float4*>(a.win)[i];
                __syncthreads();
                if (tid == 0) {
                    *s_tw = marker;
                    *s_win = a.win;
                }
            }
            FusedArgs b = a;
            b.frames = f0 + nf;  // frames past the tile belong to the next tile
            float* rows = reinterpret_cast<float*>(smem) + warp * F * RS;
            const float4* w4 = sw4;
            for (uint64_t g = f0 / F + warp; g * F < f0 + nf; g += 8) {
                if (a.outk == OUT_POWER) tpfl_group<EXP, OUT_POWER>(b, g, rows, s_tw1, s_tw2, w4, lane);
                else tpfl_group<EXP, OUT_POWER_SERIAL>(b, g, rows, s_tw1, s_tw2, w4, lane);
            }
            cp_async_wait_all();
            return;
        }
    }
    if constexpr (batch_pair_exp(EXP)) {
        if (a.outk == OUT_POWER && a.tw_pair) {
            // two frames per FFT: pairs f0/2 .. of the tile (f0 and nf are even
            // multiples of the CTA's pairs), the pair plan's tables (at 2^12 the
            // first exchange stage's twiddles and a two-level table for the
            // later ones) and the window resident behind the frame buffers
            static_assert(pair_cta_threads(EXP) == 256, "batch CTAs have 256 threads");
            constexpr int PPC = pair_ppc(EXP), BS = pair_buf_stride(EXP), T = pair_T(EXP);
            constexpr int TWN = pair_smem_tw_entries(EXP);
            const int tid = threadIdx.x;
            float2* st = reinterpret_cast<float2*>(reinterpret_cast<char*>(smem) + batch_frames_smem());
            float2* s2 = st + TWN;  // the later stages' two-level table (from 2^12)
            float* sw = reinterpret_cast<float*>(reinterpret_cast<char*>(s2) + pair_tw2l_bytes(EXP));
            const bool new_tw = *s_tw != a.tw_pair, new_win = *s_win != a.win;
            if (new_tw || new_win) {
                __syncthreads();  // the previous tile's table reads are over
                if (new_tw) {
                    for (int i = tid; i < TWN; i += 256) st[i] = a.tw_pair[i];
                    if constexpr (pair_tw2l(EXP)) {
                        // lo[e] = W_N^e (e < 128), hi[h] = W_N^(128 h), as the paired kernel builds them
                        for (int i = tid; i < 128 + (1 << EXP) / 128; i += 256) {
                            const int e = i < 128 ? i : (i - 128) * 128;
                            double sn, cs;
                            sincospi(2.0 * (double)e / (double)(1 << EXP), &sn, &cs);
                            s2[i] = make_float2((float)cs, (float)(-sn));
                        }
                    }
                }
                for (int i = tid; i < (1 << EXP); i += 256) sw[i] = a.win[i];
                __syncthreads();
                if (tid == 0) {
                    *s_tw = a.tw_pair;
                    *s_win = a.win;
                }
            }
            FusedArgs b = a;
            b.frames = f0 + nf;  // frames past the tile belong to the next tile
            b.tw = a.tw_pair;
            const int lp = tid / T, t = tid - lp * T;
            TwTwoLevel tw2{nullptr, nullptr};
            if constexpr (pair_tw2l(EXP)) tw2 = TwTwoLevel{s2, s2 + 128};
            for (uint64_t pbase = f0 / 2; 2 * pbase < f0 + nf; pbase += PPC) {
                const uint64_t q = pbase + PPC + lp;  // this group's next pair in the tile
                if (t == 0 && 2 * q < b.frames) {
                    const uint64_t s0 = 2 * q * b.hop, end = s0 + b.hop + (uint64_t)(1 << EXP);
                    prefetch_l2_span(b.x, s0, end < b.n ? end : b.n);
                }
                pair_group<EXP, OUT_POWER>(b, pbase, smem + lp * BS, smem + PPC * BS, st, tw2, sw, tid, lp, t);
            }
            return;
        }
    }
    using K = Core<EXP>;
    constexpr int T = K::T;
    constexpr int FPC = fused_fpc(EXP);
    constexpr int BS = fused_buf_stride(EXP);
    const int tid = threadIdx.x;
    const int lf = tid / T;
    const int t = tid - lf * T;
    float2* buf = smem + lf * BS;
    float* red = reinterpret_cast<float*>(smem + FPC * BS);
    const float2* tw = a.tw;
    const float2* win2 = reinterpret_cast<const float2*>(a.win);
    if constexpr (EXP <= kBatchSmemTabMaxExp) {
        constexpr int TWN = fused_tw_size(EXP);
        float2* st = reinterpret_cast<float2*>(reinterpret_cast<char*>(smem) + batch_frames_smem());
        float2* sw = st + TWN;
        // every thread sees the same pointers: uniform branches; only the
        // table that differs from the previous tile's is copied
        const bool new_tw = *s_tw != a.tw, new_win = *s_win != a.win;
        if (new_tw || new_win) {
            __syncthreads();  // the previous tile's table reads are over
            if (new_tw)
                for (int i = tid; i < TWN; i += 256) st[i] = a.tw[i];
            if (new_win || new_tw)  // the window sits behind the twiddle table
                for (int i = tid; i < (1 << EXP) / 2; i += 256) sw[i] = win2[i];
            __syncthreads();
            if (tid == 0) {
                *s_tw = a.tw;
                *s_win = a.win;
            }
        }
        tw = st;
        win2 = sw;
    }
    FusedArgs b = a;
    b.frames = f0 + nf;  // frames past the tile belong to the next tile
    // The output kind is the same for the whole tile.  Power tiles get a body
    // specialised for it, except at 2^13, where the extra body makes the
    // kernel spill under its 128-register cap; other kinds take the run-time
    // body.  (2^11 spilled too until the power body went to four bins per
    // untangle; now its power tiles run at 0.63 of HBM against 0.50 with the
    // run-time body.)
    // each frame group prefetches its next frame of the tile into L2
    auto run = [&](const auto& twx) {
        if (EXP != 13 && a.outk == OUT_POWER) {
            for (uint64_t fb = f0; fb < f0 + nf; fb += FPC) {
                fused_prefetch_next<EXP>(b, fb + FPC + lf, t);
                fused_group_frames<EXP, (EXP != 13) ? OUT_POWER : OUT_RUNTIME>(b, fb, buf, red, twx,
                                                                                             win2, tid, lf, t);
            }
        } else {
            for (uint64_t fb = f0; fb < f0 + nf; fb += FPC) {
                fused_prefetch_next<EXP>(b, fb + FPC + lf, t);
                fused_group_frames<EXP, OUT_RUNTIME>(b, fb, buf, red, twx, win2, tid, lf, t);
            }
        }
    };
    if constexpr (EXP > kBatchSmemTabMaxExp) {
        float2* st = reinterpret_cast<float2*>(reinterpret_cast<char*>(smem) + batch_frames_smem());
        if (*s_tw != a.tw || *s_win != nullptr) {
            __syncthreads();  // the previous tile's table reads are over
            build_tw2<EXP>(a.tw, st, tid, 256);
            __syncthreads();
            if (tid == 0) {
                *s_tw = a.tw;
                *s_win = nullptr;  // marks the region as holding a two-level table
            }
        }
        run(TwTwoLevel{st, st + 128});
    } else {
        run(tw);
    }
}

__global__ void __launch_bounds__(256, 2)
stft_batch_kernel(const FusedArgs* __restrict__ reqs, const BatchTile* __restrict__ tiles,
                  const uint32_t* __restrict__ ntiles, uint32_t* __restrict__ counter)
{
    extern __shared__ float2 smem[];
    __shared__ uint32_t s_tile;
    __shared__ const float2* s_tw;  // tables now in shared memory (see batch_tile)
    __shared__ const float* s_win;
    const uint32_t nt = *ntiles;
    if (threadIdx.x == 0) {
        s_tw = nullptr;
        s_win = nullptr;
        s_tile = atomicAdd(counter, 1u);
    }
    for (;;) {
        __syncthreads();  // s_tile is written; the previous tile's smem use is over
        const uint32_t ti = s_tile;
        __syncthreads();  // every thread has read s_tile
        if (ti >= nt) break;
        if (threadIdx.x == 0) {
            // claim the next tile now and start its first frames toward L2,
            // so that they arrive while this tile computes
            const uint32_t nx = atomicAdd(counter, 1u);
            s_tile = nx;
            if (nx < nt) {
                const BatchTile tn = tiles[nx];
                const FusedArgs& an = reqs[tn.req];
                const uint64_t k = tn.nframes < kBatchClaimPrefetch ? tn.nframes : kBatchClaimPrefetch;
                const uint64_t s0 = tn.f0 * an.hop, end = (tn.f0 + k - 1) * an.hop + (1ull << an.exp);
                prefetch_l2_span(an.x, s0, end < an.n ? end : an.n);
            }
        }
        const BatchTile tl = tiles[ti];
        const FusedArgs a = reqs[tl.req];
        switch (a.exp) {
        case 6: batch_tile<6>(a, tl.f0, tl.nframes, smem, &s_tw, &s_win); break;
        case 7: batch_tile<7>(a, tl.f0, tl.nframes, smem, &s_tw, &s_win); break;
        case 8: batch_tile<8>(a, tl.f0, tl.nframes, smem, &s_tw, &s_win); break;
        case 9: batch_tile<9>(a, tl.f0, tl.nframes, smem, &s_tw, &s_win); break;
        case 10: batch_tile<10>(a, tl.f0, tl.nframes, smem, &s_tw, &s_win); break;
        case 11: batch_tile<11>(a, tl.f0, tl.nframes, smem, &s_tw, &s_win); break;
        case 12: batch_tile<12>(a, tl.f0, tl.nframes, smem, &s_tw, &s_win); break;
        case 13: batch_tile<13>(a, tl.f0, tl.nframes, smem, &s_tw, &s_win); break;
        default: break;
        }
    }
}

size_t batch_smem_bytes() { return batch_smem_ct(); }
bool batch_supports(int exp) { return exp >= kBatchMinExp && exp <= kBatchMaxExp; }
// a tile is `groups` CTA-groups of frames (the host's autotuner picks the
// count per batch mix; any count keeps tiles whole groups of every body)
int batch_tile_frames(int exp, int groups) { return fused_fpc(exp) * groups; }

int batch_occupancy()
{
    int blocks = 0;
    const size_t sm = batch_smem_ct();
    if (cudaFuncSetAttribute(stft_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, stft_batch_kernel, 256, sm) != cudaSuccess) return 0;
    return blocks;
}

cudaError_t launch_batch(const FusedArgs* d_reqs, const BatchTile* d_tiles, const uint32_t* d_ntiles,
                         uint32_t* d_counter, int grid, cudaStream_t st)
{
    const size_t sm = batch_smem_ct();
    const cudaError_t e = ensure_smem_attr<stft_batch_kernel>(sm);
    if (e != cudaSuccess) return e;
    stft_batch_kernel<<<grid, 256, sm, st>>>(d_reqs, d_tiles, d_ntiles, d_counter);
    return cudaGetLastError();
}

}  // namespace ocs
