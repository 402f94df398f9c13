// A batch entry point for callers that must not allocate GPU memory.
//
// ocs_batch_device keeps its per-call scratch (request descriptors, the tile
// list and the tile-queue counter) and its plans (twiddle and window tables)
// in device memory that the library allocates on demand.  Some callers cannot
// allow that: code that owns the whole device through its own allocator,
// processes that must never block on or fail in cudaMalloc once they are
// running, or callers that have already handed every free byte to another
// pool.  ocs_batch_device_noalloc serves them.  It runs the same batch kernel
// body, and all of its scratch lives in one fixed array that is part of the
// loaded library image:
//
//     static __device__ __align__(256) unsigned char g_noalloc_scratch[1 MiB]
//
// Every GPU that loads the library holds this 1 MiB until the process exits.
// The caller passes the inputs and outputs (device pointers) as for
// ocs_batch_device.  Nothing here calls cudaMalloc, cudaFree, cudaHostAlloc or
// any other allocating CUDA routine; the host-side option parsing only uses
// small ordinary heap temporaries.
//
// Limits, rejected with OCS_ENOMEM and a message before anything is launched:
// at most kMaxRequests requests per call, window sizes 2^6 .. 2^13, and at most
// kWindowBytes of distinct window tables per call.
//
// Set-up: the first call on a device (with that device current) takes the
// array's device address with cudaGetSymbolAddress, fills the twiddle tables
// of every supported window size into it and waits for that to finish.  CUDA
// loads a library's device code lazily, so that first call is also when the
// array and this file's kernels take their device memory: a caller whose own
// allocator will reserve the device should make one call with count = 0 (it
// does the set-up and nothing else) before it does.  ocs_shutdown forgets
// the set-up, so a call after a device reset sets the device up again.
//
// Calls are not capturable into a CUDA graph (refused with OCS_EINVAL): a
// replay would upload whatever descriptors the host staging buffer holds
// then, which every later call rewrites.  ocs_batch_device is the capturable
// batch entry point.
//
// Sharing: every call uses the same array and leaves its contents behind.
// The call rewrites the descriptors and resets the tile counter to zero each
// time, so stale contents never matter, but two calls whose work overlaps on
// the GPU (different streams, no ordering between them) race on the array and
// corrupt each other's descriptors.  Order such calls on one stream or with
// events.
#include "../../include/occastft_gb300.h"
#include "ocs_host.h"
#include "stft_fused_kernel.cuh"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

namespace {

using ocs::FusedArgs;

constexpr size_t kScratchBytes = 1u << 20;  // 1 MiB per device
constexpr int kMinExp = 6;
constexpr int kMaxExp = 13;
constexpr int kMaxRequests = 256;
constexpr int kMaxDevices = 64;

struct NoallocReq {
    FusedArgs a;
    uint64_t tile_begin;  // first tile of this request in the call's tile numbering
    uint32_t tile_frames; // frames per tile
    uint32_t pad;
};

// scratch layout (bytes)
constexpr size_t kHeader = 256;  // u32 counter, u32 tiles, u32 requests
constexpr size_t kReqOff = kHeader;
constexpr size_t kReqBytes = ((sizeof(NoallocReq) * kMaxRequests + 255) / 256) * 256;
constexpr size_t tw_bytes(int e) { return ((size_t)ocs::fused_tw_size(e) * sizeof(float2) + 255) / 256 * 256; }
constexpr size_t tw_off(int e)
{
    size_t off = kReqOff + kReqBytes;
    for (int i = kMinExp; i < e; ++i) off += tw_bytes(i);
    return off;
}
constexpr size_t kWinOff = tw_off(kMaxExp + 1);
constexpr size_t kWindowBytes = kScratchBytes - kWinOff;
static_assert(kWinOff + (1u << kMaxExp) * 4 <= kScratchBytes, "scratch too small for one window table");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// host staging of the descriptors and window tables (pageable, copied at call time)
alignas(256) unsigned char g_host_stage[kScratchBytes];
std::mutex g_mu;

struct DeviceSetup {
    bool ready = false;
    unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
    int grid = 0;
};
DeviceSetup g_dev[kMaxDevices];

int fail(int code, const std::string& m)
{
    ocs::set_last_error(m);  // read back with ocs_last_error()
    return code;
}

template <int EXP>
__device__ __forceinline__ void tile_frames(const FusedArgs& a, uint64_t f0, uint32_t nf, float2* smem)
{
    using K = ocs::Core<EXP>;
    constexpr int T = K::T;
    constexpr int FPC = ocs::fused_fpc(EXP);
    constexpr int BS = ocs::fused_buf_stride(EXP);
    const int tid = threadIdx.x;
    const int lf = tid / T;
    const int t = tid - lf * T;
    float2* buf = smem + lf * BS;
    float* red = reinterpret_cast<float*>(smem + FPC * BS);
    FusedArgs b = a;
    b.frames = f0 + nf;
    for (uint64_t fb = f0; fb < f0 + nf; fb += FPC)
        ocs::fused_group_frames<EXP, ocs::OUT_RUNTIME>(b, fb, buf, red, a.tw, reinterpret_cast<const float2*>(a.win),
                                                      tid, lf, t);
}

constexpr size_t smem_bytes()
{
    size_t m = 0;
    for (int e = kMinExp; e <= kMaxExp; ++e) {
        const size_t b = (size_t)ocs::fused_fpc(e) * ocs::fused_buf_stride(e) * 8 + 8 * 4 + 16;
        m = b > m ? b : m;
    }
    return m;
}

// The batch kernel with its scratch in g_noalloc_scratch: tiles are numbered
// per call; a CTA maps its tile to a request by binary search over the
// requests' first tiles, so no tile list is stored.
__global__ void __launch_bounds__(256, 2) stft_batch_noalloc_kernel(unsigned char* scratch)
{
    extern __shared__ float2 smem[];
    __shared__ uint32_t s_tile, s_req;
    uint32_t* hdr = reinterpret_cast<uint32_t*>(scratch);
    const NoallocReq* reqs = reinterpret_cast<const NoallocReq*>(scratch + kReqOff);
    const uint32_t ntiles = hdr[1];
    const uint32_t nreq = hdr[2];
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t ti = atomicAdd(&hdr[0], 1u);
            uint32_t lo = 0, hi = nreq;  // last request with tile_begin <= ti
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) / 2;
                if (reqs[mid].tile_begin <= ti) lo = mid;
                else hi = mid;
            }
            s_tile = ti;
            s_req = lo;
        }
        __syncthreads();
        const uint32_t ti = s_tile;
        const uint32_t ri = s_req;
        __syncthreads();
        if (ti >= ntiles) break;
        const NoallocReq rq = reqs[ri];
        const uint64_t f0 = (uint64_t)(ti - rq.tile_begin) * rq.tile_frames;
        const uint32_t nf = (uint32_t)min((uint64_t)rq.tile_frames, rq.a.frames - f0);
        switch (rq.a.exp) {
        case 6: tile_frames<6>(rq.a, f0, nf, smem); break;
        case 7: tile_frames<7>(rq.a, f0, nf, smem); break;
        case 8: tile_frames<8>(rq.a, f0, nf, smem); break;
        case 9: tile_frames<9>(rq.a, f0, nf, smem); break;
        case 10: tile_frames<10>(rq.a, f0, nf, smem); break;
        case 11: tile_frames<11>(rq.a, f0, nf, smem); break;
        case 12: tile_frames<12>(rq.a, f0, nf, smem); break;
        case 13: tile_frames<13>(rq.a, f0, nf, smem); break;
        default: break;
        }
    }
}

// FP64 twiddle tables (rounded once), the same values as the cached plans
__global__ void noalloc_twiddles_kernel(float2* tw, int exp)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const ocs::FusedCfg c = ocs::fused_cfg(exp);
    const int M = 1 << (exp - 1);
    if (idx >= ocs::fused_tw_size(exp)) return;
    long long p, L;
    if (idx < M) {
        p = idx;
        L = 2LL * M;
    } else {
        int s = 1;
        while (s + 1 < c.nstages && idx >= ocs::fused_tw_offset(exp, s + 1)) ++s;
        const int e = idx - ocs::fused_tw_offset(exp, s);
        const int ns = ocs::fused_Ns(exp, s);
        p = (long long)(e % ns) * (e / ns + 1);
        L = (long long)ns * c.radix[s];
    }
    double sn, cs;
    sincospi(2.0 * (double)(p % L) / (double)L, &sn, &cs);
    tw[idx] = make_float2((float)cs, (float)(-sn));
}

// once per device, with that device current
int setup_locked(int dev, cudaStream_t st)
{
    DeviceSetup& d = g_dev[dev];
    if (d.ready) return OCS_OK;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail(OCS_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    unsigned char* scratch = static_cast<unsigned char*>(p);
    for (int x = kMinExp; x <= kMaxExp; ++x) {
        const int n = ocs::fused_tw_size(x);
        noalloc_twiddles_kernel<<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<float2*>(scratch + tw_off(x)), x);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(stft_batch_noalloc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem_bytes());
    int occ = 0, sms = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, stft_batch_noalloc_kernel, 256, smem_bytes());
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(OCS_ECUDA, std::string("no-allocation set-up: ") + cudaGetErrorString(e));
    d.scratch = scratch;
    d.grid = sms * std::max(1, occ);
    d.ready = true;
    return OCS_OK;
}

}  // namespace

namespace ocs {
namespace internal {
// Forgets the per-device set-up (called by ocs_shutdown): after a
// cudaDeviceReset the module is loaded again, possibly at another address,
// and its tables are gone, so the next call sets the device up afresh.
void noalloc_forget_devices()
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (DeviceSetup& d : g_dev) d = DeviceSetup{};
}
}  // namespace internal
}  // namespace ocs

extern "C" int ocs_batch_device_noalloc(ocs_request* reqs, int count, void* stream)
{
    if (count < 0 || (count > 0 && !reqs)) return fail(OCS_EINVAL, "bad request list");
    if (count > kMaxRequests)
        return fail(OCS_ENOMEM, "no-allocation batch: more than " + std::to_string(kMaxRequests) +
                                    " requests in one call");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // A captured call would replay its descriptor upload from the host
    // staging buffer, which every later call rewrites: refused.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing(st, &cap);
    if (ce != cudaSuccess) return fail(OCS_ECUDA, cudaGetErrorString(ce));
    if (cap != cudaStreamCaptureStatusNone)
        return fail(OCS_EINVAL, "no-allocation batch: calls cannot be captured into a CUDA graph");
    int dev = 0;
    ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return fail(OCS_ECUDA, cudaGetErrorString(ce));
    if (dev < 0 || dev >= kMaxDevices) return fail(OCS_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    int rc = setup_locked(dev, st);
    if (rc) return rc;
    unsigned char* scratch = g_dev[dev].scratch;

    // parse, validate, order by (window exponent, output kind)
    struct Item {
        int idx, exp, outk;
        ocs::Options o;
        ocs::Geometry g;
    };
    Item items[kMaxRequests];
    int ni = 0;
    for (int i = 0; i < count; ++i) {
        ocs_request& q = reqs[i];
        Item it;
        it.idx = i;
        std::string s = ocs::parse_options(q.options, it.o);
        int st_i = OCS_OK;
        if (s != "OK") {
            st_i = OCS_EPIPELINE;
        } else {
            s = ocs::make_geometry(q.n, q.window_size_exp, q.overlap_ratio, it.o, it.g);
            if (s != "OK") st_i = OCS_EINVAL;
            else if (q.window_size_exp > kMaxExp) st_i = OCS_EINVAL;
            // the tensor-core forms keep tables this array has no room for:
            // refused rather than silently run in FP32
            else if (it.o.precision != 0) st_i = OCS_EINVAL;
            else if (q.out_cap < it.g.out_floats) st_i = OCS_ESPACE;
            else if (!q.in || !q.out) st_i = OCS_EINVAL;
        }
        q.status = st_i;
        if (st_i != OCS_OK) continue;
        it.exp = q.window_size_exp;
        it.outk = it.o.half_complex ? ocs::OUT_HALF : (it.o.serial_power ? ocs::OUT_POWER_SERIAL : ocs::OUT_POWER);
        items[ni++] = it;
    }
    std::stable_sort(items, items + ni, [](const Item& a, const Item& b) {
        return a.exp != b.exp ? a.exp < b.exp : a.outk < b.outk;
    });

    // window tables (scaled by 1/2), one per distinct (kind, exponent, sigma)
    struct Win {
        int kind, exp;
        float sigma;
        size_t off;
    };
    Win wins[kMaxRequests];
    int nw = 0;
    size_t woff = kWinOff;
    NoallocReq* hreq = reinterpret_cast<NoallocReq*>(g_host_stage + kReqOff);
    uint64_t tiles = 0;
    for (int k = 0; k < ni; ++k) {
        const Item& it = items[k];
        const ocs_request& q = reqs[it.idx];
        const int kind = it.o.window;
        const float sigma = kind == ocs::WIN_GAUSSIAN ? it.o.sigma : -1.0f;
        int w = -1;
        for (int j = 0; j < nw; ++j)
            if (wins[j].kind == kind && wins[j].exp == it.exp && std::memcmp(&wins[j].sigma, &sigma, 4) == 0) w = j;
        if (w < 0) {
            const size_t bytes = ((size_t)4 << it.exp);
            if (woff + bytes > kScratchBytes) {
                // nothing is launched: no request of this call gets a result
                for (int j = 0; j < ni; ++j) reqs[items[j].idx].status = OCS_ENOMEM;
                return fail(OCS_ENOMEM, "no-allocation batch: distinct window tables exceed " +
                                            std::to_string(kWindowBytes) + " bytes");
            }
            float* dst = reinterpret_cast<float*>(g_host_stage + woff);
            if (kind == ocs::WIN_NONE) {
                for (int i = 0; i < (1 << it.exp); ++i) dst[i] = 0.5f;
            } else {
                const std::vector<float> tab = ocs::window_table(kind, 1 << it.exp, sigma);
                for (int i = 0; i < (1 << it.exp); ++i) dst[i] = tab[i] * 0.5f;
            }
            wins[nw] = Win{kind, it.exp, sigma, woff};
            w = nw++;
            woff += (bytes + 255) / 256 * 256;
        }
        NoallocReq r{};
        FusedArgs& a = r.a;
        a.x = q.in;
        a.n = q.n;
        a.hop = it.g.hop;
        a.frames = it.g.frames;
        a.win = reinterpret_cast<const float*>(scratch + wins[w].off);
        a.tw = reinterpret_cast<const float2*>(scratch + tw_off(it.exp));
        a.out = q.out;
        a.ohalf = it.o.half_complex && !it.o.dense ? it.g.ohalf : 0;
        a.dense = it.o.dense;
        a.remove_dc = it.o.remove_dc;
        a.vec2 = (it.g.hop % 2 == 0) && ((reinterpret_cast<uintptr_t>(q.in) & 7u) == 0);
        a.exp = it.exp;
        a.outk = it.outk;
        r.tile_frames = (uint32_t)ocs::fused_fpc(it.exp) * 4;
        r.tile_begin = tiles;
        tiles += (it.g.frames + r.tile_frames - 1) / r.tile_frames;
        hreq[k] = r;
    }
    if (ni == 0) return OCS_OK;
    if (tiles >= 0xffffffffull) {
        for (int j = 0; j < ni; ++j) reqs[items[j].idx].status = OCS_ENOMEM;
        return fail(OCS_ENOMEM, "no-allocation batch: too many tiles in one call");
    }
    uint32_t* hdr = reinterpret_cast<uint32_t*>(g_host_stage);
    hdr[0] = 0;  // the tile counter must start at zero on every call
    hdr[1] = (uint32_t)tiles;
    hdr[2] = (uint32_t)ni;
    // header + descriptors, then the window tables this call uses
    ce = cudaMemcpyAsync(scratch, g_host_stage, kReqOff + sizeof(NoallocReq) * ni, cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess && woff > kWinOff)
        ce = cudaMemcpyAsync(scratch + kWinOff, g_host_stage + kWinOff, woff - kWinOff, cudaMemcpyHostToDevice, st);
    if (ce != cudaSuccess) return fail(OCS_ECUDA, cudaGetErrorString(ce));
    const int grid = (int)std::min<uint64_t>((uint64_t)g_dev[dev].grid, tiles);
    stft_batch_noalloc_kernel<<<grid, 256, smem_bytes(), st>>>(scratch);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) return fail(OCS_ECUDA, cudaGetErrorString(ce));
    return OCS_OK;
}
