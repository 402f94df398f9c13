// C ABI of the GB300 STFT runner (include/occastft_gb300.h).
//
// Replaces the CUDA vendor runner of OCCAstft
// (StandAlone/cross_gpgpu/CUDA/src/CudaImpl.cpp, functionImpl.cpp): where the
// reference allocates, copies, runs 7+ kernels, copies back and frees on
// every request, this runner keeps per-exponent plans (twiddle tables built
// once in FP64 on the device, window tables built once on the host) and
// request slots (streams + grow-only device buffers) resident, runs the
// whole pipeline as one fused kernel, and overlaps host->device copies,
// compute and device->host copies across frame chunks.
#include "../../include/occastft_gb300.h"
#include "ocs_host.h"
#include "ocs_internal.h"
#include "ocs_kernels.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* where)
{
    return fail(OCS_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define OCS_CUDA(call)                                          \
    do {                                                        \
        cudaError_t _e = (call);                                \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);     \
    } while (0)

struct Slot {
    cudaStream_t s_h2d = nullptr, s_comp = nullptr, s_d2h = nullptr;
    std::vector<cudaEvent_t> ev_in, ev_comp;
    float* d_in = nullptr;
    size_t in_cap = 0;   // floats
    float* d_out = nullptr;
    size_t out_cap = 0;  // floats
};

// at most 16 chunks per ocs_activate call: at 1e8 samples 4, 8 or 25 MB of
// input per chunk measured the same end to end (20.8-21.6 Gsamples/s; the
// host link, not the pipeline's fill and drain, sets the time)
constexpr int kMaxChunks = 16;

struct Context {
    std::mutex mu;
    bool ready = false;
    int device = -1;
    int sms = 0;
    cudaStream_t s_setup = nullptr;
    std::map<int, float2*> twiddles;                             // exp * 2 + paired -> table
    std::map<std::tuple<int, int, uint32_t>, float*> windows;    // (kind, exp, sigma bits) -> table
    std::map<const float*, std::vector<float>> windows_host;     // device table -> host copy (windows <= 2^8)
    std::map<uint64_t, float2*> two_level;                       // L -> exp(-2 pi i j / L) lo|hi table
    std::map<std::pair<int, int>, int> occupancy;                // (exp, output kind) -> CTAs per SM
    std::vector<Slot*> free_slots;
    std::vector<Slot*> all_slots;
    std::map<std::tuple<int, int, int, int>, int> tuned;          // (exp, outk, dense, log2 frames) -> variant
    std::map<std::pair<uint32_t, int>, int> batch_tuned;          // (window exps present, log2 frames) -> groups per tile
    // uneven batches: the scratch of ocs_batch_device
    std::mutex batch_mu;
    ocs::internal::BatchScratch batch;
    int batch_occ = 0;
    // A captured batch replays its descriptor upload from the buffers it was
    // captured with, so each capture gets its own: ocs_batch_prepare sets one
    // set aside, the next captured ocs_batch_device takes it, and it is kept
    // (with that graph's descriptors) until ocs_shutdown.
    ocs::internal::BatchScratch* graph_next = nullptr;
    std::vector<ocs::internal::BatchScratch*> graph_kept;
    // error word of the bounded waits in the tensor-core kernels: mapped host
    // memory, so the host reads it without a copy or a stream order
    int* h_err = nullptr;
    int* d_err = nullptr;
    int tc_test_stall = 0;  // OCS_TC_TEST_STALL=1: the kernel's first input phase never completes
    bool tune_loaded = false;
    std::string gpu_name;
};

Context& ctx()
{
    static Context* c = new Context();  // never destroyed: outlives static teardown order
    return *c;
}

int init_locked(Context& c, int device)
{
    if (c.ready) {
        if (device >= 0 && device != c.device) return fail(OCS_EINVAL, "ocs_init: already initialised on another device");
        OCS_CUDA(cudaSetDevice(c.device));
        return OCS_OK;
    }
    if (device < 0) OCS_CUDA(cudaGetDevice(&device));
    OCS_CUDA(cudaSetDevice(device));
    cudaDeviceProp p;
    OCS_CUDA(cudaGetDeviceProperties(&p, device));
    if (p.major < 10) return fail(OCS_EINVAL, "this runner is built for sm_103a (Blackwell Ultra)");
    c.device = device;
    c.sms = p.multiProcessorCount;
    c.gpu_name = p.name;
    cudaError_t e = cudaStreamCreateWithFlags(&c.s_setup, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaHostAlloc(&c.h_err, sizeof(int), cudaHostAllocMapped);
    if (e == cudaSuccess) {
        *reinterpret_cast<volatile int*>(c.h_err) = 0;
        e = cudaHostGetDevicePointer(&c.d_err, c.h_err, 0);
    }
    if (e != cudaSuccess) {  // a later call starts over from nothing
        if (c.h_err) cudaFreeHost(c.h_err);
        if (c.s_setup) cudaStreamDestroy(c.s_setup);
        c.h_err = nullptr;
        c.d_err = nullptr;
        c.s_setup = nullptr;
        return cuda_fail(e, "runner set-up");
    }
    const char* stall = std::getenv("OCS_TC_TEST_STALL");
    c.tc_test_stall = (stall && stall[0] == '1') ? 1 : 0;
    c.ready = true;
    return OCS_OK;
}

// Reads and clears the tensor-core error word.  The kernels write it
// directly into mapped host memory, so once their stream has been
// synchronised the value is current.
int take_tc_error()
{
    Context& c = ctx();
    if (!c.h_err) return OCS_OK;
    volatile int* w = reinterpret_cast<volatile int*>(c.h_err);
    if (*w == 0) return OCS_OK;
    *w = 0;
    return fail(OCS_ETIMEDOUT, "tensor-core kernel: a pipeline wait gave up after one second");
}

int ensure_init()
{
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    return init_locked(c, c.ready ? c.device : -1);
}

// exp: the window exponent, or the plan id of a paired table
int get_twiddles(int exp, bool paired, const float2** out)
{
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    const int key = exp * 2 + (paired ? 1 : 0);
    auto it = c.twiddles.find(key);
    if (it != c.twiddles.end()) {
        *out = it->second;
        return OCS_OK;
    }
    float2* d = nullptr;
    const int n = paired ? ocs::pair_twiddle_count(exp) : ocs::fused_twiddle_count(exp);
    OCS_CUDA(cudaMalloc(&d, sizeof(float2) * n));
    cudaError_t e = paired ? ocs::build_pair_twiddles(d, exp, c.s_setup) : ocs::build_twiddles(d, exp, c.s_setup);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.s_setup);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "twiddle table");
    }
    c.twiddles[key] = d;
    *out = d;
    return OCS_OK;
}

// Window table of (kind, exp, sigma).  scaled = true gives the table the fused
// kernels consume: coefficients times 1/2 (exact), all 1/2 for no window.
int get_window(int kind, int exp, float sigma, bool scaled, const float** out)
{
    *out = nullptr;
    if (kind == ocs::WIN_NONE && !scaled) return OCS_OK;
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    uint32_t sbits = 0;
    if (kind == ocs::WIN_GAUSSIAN) std::memcpy(&sbits, &sigma, 4);
    const auto key = std::make_tuple(kind * 2 + (scaled ? 1 : 0), exp, sbits);
    auto it = c.windows.find(key);
    if (it != c.windows.end()) {
        *out = it->second;
        return OCS_OK;
    }
    std::vector<float> w = ocs::window_table(kind, 1 << exp, sigma);
    if (kind == ocs::WIN_NONE) w.assign((size_t)1 << exp, 1.0f);
    if (scaled)
        for (float& v : w) v *= 0.5f;
    float* d = nullptr;
    OCS_CUDA(cudaMalloc(&d, sizeof(float) * w.size()));
    cudaError_t e = cudaMemcpyAsync(d, w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice, c.s_setup);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.s_setup);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(e, "window table");
    }
    c.windows[key] = d;
    if (exp <= 8) c.windows_host[d] = w;  // the lanes-per-frame kernels take it as a parameter
    *out = d;
    return OCS_OK;
}

// Host copy of a window table that get_window made (windows up to 2^8), or null.
const float* host_window(const float* d)
{
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    auto it = c.windows_host.find(d);
    return it == c.windows_host.end() ? nullptr : it->second.data();
}

// ---------------------------------------------------------------- kernel choice
// Variants of the fused kernel: 0 one frame per FFT, direct I/O; 1 one frame
// per FFT, shared-memory staged I/O (windows <= 2^9); 2 two frames per FFT;
// 3 N/64 lanes per frame, the FFT in registers (windows 2^6 .. 2^8 for power,
// 2^6 for half-complex); 4 two frames per FFT on packed FP32x2 arithmetic
// (window 2^10).
enum { VAR_DIRECT = 0, VAR_STAGED = 1, VAR_PAIR = 2, VAR_TPF = 3, VAR_PAIRX2 = 4, VAR_COUNT = 5 };

bool env_is(const char* name, const char* val)
{
    const char* e = std::getenv(name);
    return e && std::strcmp(e, val) == 0;
}

// defaults measured on GB300 (1e8 samples, overlap 0.5, the autotuner's own
// picks) for when tuning is off or the stream is being captured
int default_variant(int exp, int outk)
{
    const bool power = outk != ocs::OUT_HALF;
    if (power) {
        if (exp <= 8) return VAR_TPF;
        if (exp == 10) return VAR_PAIRX2;
        if (exp == 9 || exp == 12 || exp == 13 || exp == 14) return VAR_PAIR;
        return VAR_DIRECT;
    }
    if (exp == 6) return VAR_TPF;
    if (exp == 14) return VAR_PAIR;
    return VAR_DIRECT;
}
bool variant_ok(int v, int exp, int outk, bool out16)
{
    if (v == VAR_PAIRX2)
        return ocs::pairx2_has(exp, outk) && !env_is("OCS_KERNEL", "single") && !env_is("OCS_KERNEL", "pair");
    if (v == VAR_PAIR) return ocs::pair_has(exp) && outk != ocs::OUT_PLANES && !env_is("OCS_KERNEL", "single");
    if (v == VAR_STAGED)
        return ocs::fused_has_staged(exp) && outk != ocs::OUT_PLANES && out16 && !env_is("OCS_IO_SCHEME", "direct");
    if (v == VAR_TPF)
        return ocs::tpf_has(exp, outk) && out16 && !env_is("OCS_IO_SCHEME", "direct") && !env_is("OCS_KERNEL", "single");
    return true;
}

std::string tune_cache_path()
{
    const char* e = std::getenv("OCS_TUNE_CACHE");
    return e ? std::string(e) : std::string();
}

// tuning cache file: one "gpu|exp|outk|dense|bucket|variant" line per entry
void tune_load_locked(Context& c)
{
    if (c.tune_loaded) return;
    c.tune_loaded = true;
    const std::string path = tune_cache_path();
    if (path.empty()) return;
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return;
    char line[512];
    while (std::fgets(line, sizeof line, f)) {
        char name[256];
        int e, o, d, b, v;
        if (std::sscanf(line, "%255[^|]|%d|%d|%d|%d|%d", name, &e, &o, &d, &b, &v) == 6 && c.gpu_name == name)
            c.tuned[std::make_tuple(e, o, d, b)] = v;
    }
    std::fclose(f);
}

void tune_store_locked(Context& c, const std::tuple<int, int, int, int>& k, int v)
{
    c.tuned[k] = v;
    const std::string path = tune_cache_path();
    if (path.empty()) return;
    FILE* f = std::fopen(path.c_str(), "a");
    if (!f) return;
    std::fprintf(f, "%s|%d|%d|%d|%d|%d\n", c.gpu_name.c_str(), std::get<0>(k), std::get<1>(k), std::get<2>(k),
                 std::get<3>(k), v);
    std::fclose(f);
}

int grid_size(int exp, int outk, int variant, uint64_t frames)
{
    Context& c = ctx();
    int occ;
    {
        std::lock_guard<std::mutex> lk(c.mu);
        auto key = std::make_pair(exp, outk * VAR_COUNT + variant);
        auto it = c.occupancy.find(key);
        if (it == c.occupancy.end()) {
            occ = std::max(1, variant == VAR_PAIR     ? ocs::pair_occupancy(exp, outk)
                              : variant == VAR_PAIRX2 ? ocs::pairx2_occupancy(exp, outk)
                              : variant == VAR_TPF    ? ocs::tpf_occupancy(exp, outk)
                                                      : ocs::fused_occupancy(exp, outk, variant == VAR_STAGED));
            c.occupancy[key] = occ;
        } else {
            occ = it->second;
        }
    }
    const uint64_t fpc = (uint64_t)(variant == VAR_PAIR     ? 2 * ocs::pair_per_cta(exp)
                                    : variant == VAR_PAIRX2 ? 2 * ocs::pairx2_per_cta(exp)
                                    : variant == VAR_TPF    ? ocs::tpf_frames_per_cta(exp)
                                                            : ocs::fused_frames_per_cta(exp));
    const uint64_t need = (frames + fpc - 1) / fpc;
    const uint64_t full = (uint64_t)c.sms * occ;
    return (int)std::max<uint64_t>(1, std::min(need, full));
}

struct Request {
    ocs::Options opt;
    ocs::Geometry geo;
    int exp = 0;
};

int prepare(uint64_t n, int exp, float ov, const char* options, Request& r)
{
    std::string st = ocs::parse_options(options, r.opt);
    if (st != "OK") return fail(OCS_EPIPELINE, st);
    st = ocs::make_geometry(n, exp, ov, r.opt, r.geo);
    if (st != "OK") return fail(OCS_EINVAL, st);
    if (r.opt.precision >= 1 && !ocs::tc_supports(exp))
        return fail(OCS_EINVAL, "the tensor-core form supports windows 2^8 .. 2^12");
    if (r.opt.precision >= 1 && !ocs::tc_mode_supported(exp, r.opt.precision))
        return fail(OCS_EINVAL, "this tensor-core split mode is not available at this window size");
    if (r.opt.precision >= 2 && !ocs::tc_piped(exp, r.geo.hop))
        return fail(OCS_EINVAL, "the bf16 tensor-core forms need a frame advance of at most the window");
    r.exp = exp;
    return OCS_OK;
}

// the variant this thread launched last (ocs_plan_tune reports it)
thread_local int g_last_variant = -1;

cudaError_t launch_variant(int v, const Request& r, int outk, ocs::FusedArgs a, const float2* tw_single,
                           const float2* tw_pair, cudaStream_t st)
{
    g_last_variant = v;
    if (v == VAR_PAIR) {
        a.tw = tw_pair;
        return ocs::launch_pair(r.exp, outk, a, grid_size(r.exp, outk, VAR_PAIR, a.frames), st);
    }
    if (v == VAR_PAIRX2) {
        a.tw = tw_pair;
        return ocs::launch_pairx2(r.exp, outk, a, grid_size(r.exp, outk, VAR_PAIRX2, a.frames), st);
    }
    if (v == VAR_TPF) {
        const float* hw = host_window(a.win);
        if (!hw) return cudaErrorInvalidValue;
        return ocs::launch_tpf(r.exp, outk, a, hw, grid_size(r.exp, outk, VAR_TPF, a.frames), st);
    }
    a.tw = tw_single;
    return ocs::launch_fused(r.exp, outk, v == VAR_STAGED, a, grid_size(r.exp, outk, v, a.frames), st);
}

int ilog2u(uint64_t v)
{
    int l = 0;
    while (v > 1) {
        v >>= 1;
        ++l;
    }
    return l;
}

// exp(-2 pi i j / L) for j < L as lo[j % 1024] * hi[j / 1024]: 1024 + L/1024 entries
int get_two_level(uint64_t L, const float2** lo, const float2** hi)
{
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    auto it = c.two_level.find(L);
    if (it == c.two_level.end()) {
        float2* d = nullptr;
        const uint64_t nhi = (L + 1023) / 1024;
        OCS_CUDA(cudaMalloc(&d, sizeof(float2) * (1024 + nhi)));
        cudaError_t e = ocs::build_two_level(d, d + 1024, L, c.s_setup);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.s_setup);
        if (e != cudaSuccess) {
            cudaFree(d);
            return cuda_fail(e, "two-level twiddle table");
        }
        it = c.two_level.emplace(L, d).first;
    }
    *lo = it->second;
    *hi = it->second + 1024;
    return OCS_OK;
}

// Windows 2^16 .. 2^30: the four-step FFT (two launches up to 2^22, three
// above) over frames [f0, f1), with stream-ordered scratch of at most ~1 GB
// per buffer (frames in chunks; one frame at a time when a frame needs more).
// win: the scaled window table, or null for no window (the stage hook);
// out_im: the imaginary plane for the planes output.
int launch_large_core(int exp, int outk, const float* d_sig, uint64_t n, uint64_t hop, const float* win, int dense,
                      int remove_dc, uint64_t ohalf, float* d_out, float* d_out_im, uint64_t f0, uint64_t f1,
                      cudaStream_t st)
{
    if (f1 <= f0) return OCS_OK;
    const ocs::LargePlan pl = ocs::large_plan(exp);
    if (pl.passes == 0) return fail(OCS_EINVAL, "no four-step plan for this window size");
    ocs::LargeArgs a{};
    int rc = get_twiddles(pl.l1 + 1, false, &a.tw1);
    if (!rc) rc = get_twiddles(pl.l3 + 1, false, &a.tw2);
    if (!rc && pl.passes == 3) rc = get_twiddles(pl.l2 + 1, false, &a.tw3);
    const uint64_t N = 1ull << exp, M = N / 2;
    if (!rc) rc = get_two_level(M, &a.twm_lo, &a.twm_hi);
    if (!rc) rc = get_two_level(N, &a.twn_lo, &a.twn_hi);
    if (rc) return rc;
    a.x = d_sig;
    a.n = n;
    a.hop = hop;
    a.frames_total = f1;
    a.win = win;
    a.out = d_out;
    a.out_im = d_out_im;
    a.ohalf = ohalf;
    a.dense = dense;
    a.remove_dc = remove_dc;
    // scratch per chunk (OCS_LARGE_SCRATCH_MB overrides).  Measured on GB300
    // at 1e8 samples: chunks small enough for the scratch to stay in L2
    // (16-96 MB) lose to fewer, fuller launch pairs; 1 GB is the default
    uint64_t scratch_bytes = 1024ull << 20;
    if (const char* sb = std::getenv("OCS_LARGE_SCRATCH_MB"))
        scratch_bytes = (uint64_t)std::min(std::max(1L, std::atol(sb)), 1L << 20) << 20;  // 1 MB .. 1 TB
    const uint64_t per = std::max<uint64_t>(1, std::min<uint64_t>(f1 - f0, scratch_bytes / (M * sizeof(float2))));
    float2* scratch = nullptr;
    float2* scratch2 = nullptr;
    OCS_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&scratch), per * M * sizeof(float2), st));
    cudaError_t e = cudaSuccess;
    if (pl.passes == 3) e = cudaMallocAsync(reinterpret_cast<void**>(&scratch2), per * M * sizeof(float2), st);
    a.scratch = scratch;
    a.scratch2 = scratch2;
    for (uint64_t c0 = f0; c0 < f1 && e == cudaSuccess; c0 += per) {
        a.f0 = c0;
        e = ocs::launch_large(exp, outk, a, std::min(per, f1 - c0), st);
    }
    const cudaError_t e2b = cudaFreeAsync(scratch, st);
    const cudaError_t e3b = scratch2 ? cudaFreeAsync(scratch2, st) : cudaSuccess;
    if (e != cudaSuccess) return cuda_fail(e, "large-window launch");
    if (e2b != cudaSuccess) return cuda_fail(e2b, "large-window scratch");
    if (e3b != cudaSuccess) return cuda_fail(e3b, "large-window scratch");
    return OCS_OK;
}

int launch_large_frames(const Request& r, const float* d_sig, uint64_t n, float* d_out, uint64_t f0, uint64_t f1,
                        cudaStream_t st)
{
    if (f1 <= f0) return OCS_OK;
    const float* win = nullptr;
    int rc = get_window(r.opt.window, r.exp, r.opt.sigma, true, &win);
    if (rc) return rc;
    const int outk = r.opt.half_complex ? ocs::OUT_HALF : (r.opt.serial_power ? ocs::OUT_POWER_SERIAL : ocs::OUT_POWER);
    return launch_large_core(r.exp, outk, d_sig, n, r.geo.hop, win, r.opt.dense, r.opt.remove_dc,
                             r.opt.half_complex && !r.opt.dense ? (uint64_t)r.geo.ohalf : 0, d_out, nullptr, f0, f1,
                             st);
}

// Launch the fused kernel for frames [f0, f1) of a request.  The first launch
// of a new (window, output kind, layout, size class) measures every kernel
// variant that applies on the request's own buffers and keeps the fastest
// (OCS_AUTOTUNE=0 disables this; OCS_TUNE_CACHE=<file> persists choices).
int launch_frames(const Request& r, const float* d_sig, uint64_t n, float* d_out, uint64_t f0, uint64_t f1,
                  cudaStream_t st)
{
    if (ocs::large_supports(r.exp)) return launch_large_frames(r, d_sig, n, d_out, f0, f1, st);
    const float2* tw_single = nullptr;
    const float2* tw_pair = nullptr;
    const float* win = nullptr;
    int rc = get_twiddles(r.exp, false, &tw_single);
    if (rc) return rc;
    if (ocs::pair_has(r.exp)) {
        // the one-request kernels' paired plan (the batch's may differ)
        rc = get_twiddles(ocs::pair_plan_id(r.exp), true, &tw_pair);
        if (rc) return rc;
    }
    rc = get_window(r.opt.window, r.exp, r.opt.sigma, true, &win);
    if (rc) return rc;
    const uint64_t N = r.geo.n_window;
    const uint64_t hop = r.geo.hop;
    const uint64_t start = f0 * hop;
    ocs::FusedArgs a{};
    a.x = d_sig + std::min<uint64_t>(start, n);
    a.n = start < n ? n - start : 0;
    a.hop = hop;
    a.frames = f1 - f0;
    a.win = win;
    const int outk = r.opt.half_complex ? ocs::OUT_HALF : (r.opt.serial_power ? ocs::OUT_POWER_SERIAL : ocs::OUT_POWER);
    a.dense = r.opt.dense;
    a.remove_dc = r.opt.remove_dc;
    if (r.opt.dense) {
        const uint64_t row = (N / 2 + 1) * (r.opt.half_complex ? 2 : 1);
        a.out = d_out + f0 * row;
        a.ohalf = 0;
    } else if (r.opt.half_complex) {
        a.out = d_out + 2 * f0 * N;
        a.ohalf = (uint64_t)r.geo.ohalf - f0 * N;
    } else {
        a.out = d_out + f0 * N;
        a.ohalf = 0;
    }
    if (a.frames == 0) return OCS_OK;
    if (start >= n) {
        // frames entirely past the signal end still produce (zero) output
        a.x = d_sig;
        a.n = 0;
    }
    const uintptr_t xa = reinterpret_cast<uintptr_t>(a.x);
    a.vec2 = (hop % 2 == 0) && ((xa & 7u) == 0);
    a.cs = ((hop % 4 == 0) && (xa & 15u) == 0) ? 16 : (a.vec2 ? 8 : 4);
    const bool out16 = (reinterpret_cast<uintptr_t>(a.out) & 15u) == 0;

    if (r.opt.precision >= 1) {
        // tensor-core form: unscaled window (no real-input untangle)
        const float* w1 = nullptr;
        rc = get_window(r.opt.window, r.exp, r.opt.sigma, false, &w1);
        if (rc) return rc;
        a.win = w1;
        Context& c = ctx();
        OCS_CUDA(ocs::launch_tc(r.exp, outk, r.opt.precision, a, c.d_err, c.tc_test_stall, c.sms, st));
        return OCS_OK;
    }

    int cand[VAR_COUNT], nc = 0;
    for (int v = 0; v < VAR_COUNT; ++v)
        if (variant_ok(v, r.exp, outk, out16)) cand[nc++] = v;
    if (env_is("OCS_KERNEL", "tpf") && variant_ok(VAR_TPF, r.exp, outk, out16)) {
        OCS_CUDA(launch_variant(VAR_TPF, r, outk, a, tw_single, tw_pair, st));
        return OCS_OK;
    }
    if (env_is("OCS_KERNEL", "x2") && variant_ok(VAR_PAIRX2, r.exp, outk, out16)) {
        OCS_CUDA(launch_variant(VAR_PAIRX2, r, outk, a, tw_single, tw_pair, st));
        return OCS_OK;
    }
    if (env_is("OCS_KERNEL", "pair") && variant_ok(VAR_PAIR, r.exp, outk, out16)) {
        OCS_CUDA(launch_variant(VAR_PAIR, r, outk, a, tw_single, tw_pair, st));
        return OCS_OK;
    }
    int choice = default_variant(r.exp, outk);
    bool have = false;
    for (int i = 0; i < nc; ++i) have |= cand[i] == choice;
    if (!have) choice = cand[0];

    const auto key = std::make_tuple(r.exp, outk, (int)r.opt.dense, ilog2u(a.frames));
    bool need_tune = false;
    if (nc > 1 && !env_is("OCS_AUTOTUNE", "0")) {
        Context& c = ctx();
        std::lock_guard<std::mutex> lk(c.mu);
        tune_load_locked(c);
        auto it = c.tuned.find(key);
        if (it != c.tuned.end()) {
            bool ok = false;
            for (int i = 0; i < nc; ++i) ok |= cand[i] == it->second;
            if (ok) choice = it->second;
        } else {
            need_tune = true;
        }
    }
    if (need_tune) {
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(st, &cap);
        if (cap == cudaStreamCaptureStatusNone) {
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            cudaError_t te = cudaEventCreate(&e0);
            if (te == cudaSuccess) te = cudaEventCreate(&e1);
            float best = 1e30f;
            for (int i = 0; i < nc && te == cudaSuccess; ++i) {
                const int v = cand[i];
                te = launch_variant(v, r, outk, a, tw_single, tw_pair, st);
                if (te == cudaSuccess) te = cudaEventRecord(e0, st);
                for (int k = 0; k < 3 && te == cudaSuccess; ++k)
                    te = launch_variant(v, r, outk, a, tw_single, tw_pair, st);
                if (te == cudaSuccess) te = cudaEventRecord(e1, st);
                if (te == cudaSuccess) te = cudaEventSynchronize(e1);
                float ms = 0.0f;
                if (te == cudaSuccess) te = cudaEventElapsedTime(&ms, e0, e1);
                if (te == cudaSuccess && ms < best) {
                    best = ms;
                    choice = v;
                }
            }
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            if (te != cudaSuccess) return cuda_fail(te, "kernel variant timing");
            Context& c = ctx();
            std::lock_guard<std::mutex> lk(c.mu);
            tune_store_locked(c, key, choice);
        }
    }
    OCS_CUDA(launch_variant(choice, r, outk, a, tw_single, tw_pair, st));
    return OCS_OK;
}

// output floats of frames [f0, f1)
void out_range(const Request& r, uint64_t f0, uint64_t f1, uint64_t* off, uint64_t* cnt)
{
    const uint64_t N = r.geo.n_window;
    if (r.opt.dense) {
        const uint64_t row = (N / 2 + 1) * (r.opt.half_complex ? 2 : 1);
        *off = f0 * row;
        *cnt = (f1 - f0) * row;
    } else if (r.opt.half_complex) {
        const uint64_t lim = 2ull * r.geo.ohalf;
        const uint64_t a = std::min(2 * f0 * N, lim), b = std::min(2 * f1 * N, lim);
        *off = a;
        *cnt = b - a;
    } else {
        *off = f0 * N;
        *cnt = (f1 - f0) * N;
    }
}

void destroy_slot(Slot* s)
{
    if (s->s_h2d) cudaStreamDestroy(s->s_h2d);
    if (s->s_comp) cudaStreamDestroy(s->s_comp);
    if (s->s_d2h) cudaStreamDestroy(s->s_d2h);
    for (auto e : s->ev_in) cudaEventDestroy(e);
    for (auto e : s->ev_comp) cudaEventDestroy(e);
    if (s->d_in) cudaFree(s->d_in);
    if (s->d_out) cudaFree(s->d_out);
    delete s;
}

Slot* acquire_slot(int* rc)
{
    Context& c = ctx();
    {
        std::lock_guard<std::mutex> lk(c.mu);
        if (!c.free_slots.empty()) {
            Slot* s = c.free_slots.back();
            c.free_slots.pop_back();
            return s;
        }
    }
    Slot* s = new Slot();
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_h2d, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_comp, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_d2h, cudaStreamNonBlocking);
    for (int i = 0; i < kMaxChunks && e == cudaSuccess; ++i) {
        cudaEvent_t a = nullptr, b = nullptr;
        e = cudaEventCreateWithFlags(&a, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b, cudaEventDisableTiming);
        if (e == cudaSuccess) {
            s->ev_in.push_back(a);
            s->ev_comp.push_back(b);
        } else if (a) {
            cudaEventDestroy(a);
        }
    }
    if (e != cudaSuccess) {
        *rc = cuda_fail(e, "slot creation");
        destroy_slot(s);
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(c.mu);
    c.all_slots.push_back(s);
    return s;
}

void release_slot(Slot* s)
{
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    c.free_slots.push_back(s);
}

int grow(float** p, size_t* cap, size_t need)
{
    if (*cap >= need) return OCS_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(p, need * sizeof(float));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(OCS_ENOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
    }
    *cap = need;
    return OCS_OK;
}

}  // namespace


// ---------------------------------------------------------------- batches
namespace {

struct BatchPlan {
    std::vector<ocs::FusedArgs> descs;   // one per request in the persistent launch
    std::vector<ocs::BatchTile> tiles;
    std::vector<int> big;                // requests with windows above the batch kernel's range
    std::vector<Request> parsed;
};

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Parses every request, builds plans, descriptors and the ordered tile list.
int batch_build(ocs_request* reqs, int count, BatchPlan& bp, bool write_status)
{
    bp.parsed.assign(count, Request{});
    std::vector<int> order;
    for (int i = 0; i < count; ++i) {
        ocs_request& q = reqs[i];
        Request& r = bp.parsed[i];
        int rc = prepare(q.n, q.window_size_exp, q.overlap_ratio, q.options, r);
        if (!rc && q.out_cap < r.geo.out_floats) rc = fail(OCS_ESPACE, "output buffer too small");
        if (!rc && (!q.in || !q.out)) rc = fail(OCS_EINVAL, "null buffer");
        if (!rc) {
            const float2* tw = nullptr;
            const float* win = nullptr;
            rc = get_twiddles(r.exp, false, &tw);
            if (!rc) rc = get_window(r.opt.window, r.exp, r.opt.sigma, true, &win);
            if (!rc && ocs::pair_has(r.exp)) {
                const float2* twp = nullptr;
                rc = get_twiddles(r.exp, true, &twp);
            }
        }
        // the tensor-core forms build their DFT tables before a capture can need them
        if (!rc && r.opt.precision >= 1) {
            const cudaError_t te = ocs::tc_prepare(r.exp, r.opt.precision);
            if (te != cudaSuccess) rc = cuda_fail(te, "tensor-core tables");
        }
        if (write_status) q.status = rc;
        if (rc) continue;
        // requests that ask for a tensor-core precision get their own launch
        // of that form (the batch kernel is the FP32 form), as do windows
        // above the batch kernel's range
        if (ocs::batch_supports(r.exp) && r.opt.precision == 0) order.push_back(i);
        else bp.big.push_back(i);
    }
    auto outk_of = [&](int i) {
        const Request& r = bp.parsed[i];
        return r.opt.half_complex ? ocs::OUT_HALF : (r.opt.serial_power ? ocs::OUT_POWER_SERIAL : ocs::OUT_POWER);
    };
    // tiles ordered by (window size, output kind, window table): a CTA's
    // successive tiles then mostly share one code path and one window table,
    // which the batch kernel keeps in shared memory between tiles
    auto win_key = [&](int i) {
        const Request& r = bp.parsed[i];
        uint32_t sb;
        std::memcpy(&sb, &r.opt.sigma, sizeof sb);
        return std::make_tuple(r.opt.window, sb);
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const int ea = bp.parsed[a].exp, eb = bp.parsed[b].exp;
        if (ea != eb) return ea < eb;
        if (outk_of(a) != outk_of(b)) return outk_of(a) < outk_of(b);
        return win_key(a) < win_key(b);
    });
    for (int i : order) {
        const Request& r = bp.parsed[i];
        const ocs_request& q = reqs[i];
        ocs::FusedArgs a{};
        const float2* tw = nullptr;
        const float* win = nullptr;
        get_twiddles(r.exp, false, &tw);
        get_window(r.opt.window, r.exp, r.opt.sigma, true, &win);
        a.x = q.in;
        a.n = q.n;
        a.hop = r.geo.hop;
        a.frames = r.geo.frames;
        a.win = win;
        a.tw = tw;
        if (ocs::pair_has(r.exp)) get_twiddles(r.exp, true, &a.tw_pair);
        a.out = q.out;
        a.ohalf = r.opt.half_complex && !r.opt.dense ? r.geo.ohalf : 0;
        a.dense = r.opt.dense;
        a.remove_dc = r.opt.remove_dc;
        a.vec2 = (r.geo.hop % 2 == 0) && ((reinterpret_cast<uintptr_t>(q.in) & 7u) == 0);
        // bytes per async copy of the lanes-per-frame tiles (2^7, 2^8 power)
        a.cs = ((r.geo.hop % 4 == 0) && (reinterpret_cast<uintptr_t>(q.in) & 15u) == 0) ? 16 : (a.vec2 ? 8 : 4);
        a.exp = r.exp;
        a.outk = outk_of(i);
        bp.descs.push_back(a);
    }
    return OCS_OK;
}

// Tile lengths the batch autotuner tries, in CTA-groups of frames per tile:
// longer tiles mean fewer queue pulls and block barriers, shorter ones a
// shorter tail.  16 is the default (measured best on average over mixes).
constexpr int kBatchGroups[] = {8, 16, 32, 64};
constexpr int kBatchGroupsDefault = 16;
constexpr int kBatchGroupsMin = 8;

// cuts every descriptor's frames into tiles of `groups` CTA-groups
void batch_tiles(BatchPlan& bp, int groups)
{
    bp.tiles.clear();
    for (uint32_t idx = 0; idx < (uint32_t)bp.descs.size(); ++idx) {
        const ocs::FusedArgs& a = bp.descs[idx];
        const uint64_t tf = (uint64_t)ocs::batch_tile_frames(a.exp, groups);
        for (uint64_t f0 = 0; f0 < a.frames; f0 += tf) {
            ocs::BatchTile t;
            t.req = idx;
            t.nframes = (uint32_t)std::min<uint64_t>(tf, a.frames - f0);
            t.f0 = f0;
            bp.tiles.push_back(t);
        }
    }
}

// the autotuner's key for a batch: which window sizes it holds and its size
std::pair<uint32_t, int> batch_mix_key(const BatchPlan& bp)
{
    uint32_t mask = 0;
    uint64_t frames = 0;
    for (const ocs::FusedArgs& a : bp.descs) {
        mask |= 1u << a.exp;
        frames += a.frames;
    }
    return std::make_pair(mask, ilog2u(frames));
}

size_t batch_bytes(size_t ndesc, size_t ntiles)
{
    return align256(ndesc * sizeof(ocs::FusedArgs)) + align256(ntiles * sizeof(ocs::BatchTile)) + 256;
}

int batch_occ_get()
{
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    if (!c.batch_occ) c.batch_occ = std::max(1, ocs::batch_occupancy());
    return c.batch_occ;
}

}  // namespace

namespace ocs {
namespace internal {

int batch_scratch_grow(BatchScratch& b, size_t bytes)
{
    if (b.host_cap < bytes) {
        if (b.staged) OCS_CUDA(cudaEventSynchronize(b.staged));
        if (b.host) cudaFreeHost(b.host);
        b.host = nullptr;
        b.host_cap = 0;
        OCS_CUDA(cudaHostAlloc((void**)&b.host, bytes, cudaHostAllocPortable));
        b.host_cap = bytes;
    }
    if (b.dev_cap < bytes) {
        if (b.done) OCS_CUDA(cudaEventSynchronize(b.done));
        if (b.dev) cudaFree(b.dev);
        b.dev = nullptr;
        b.dev_cap = 0;
        OCS_CUDA(cudaMalloc((void**)&b.dev, bytes));
        b.dev_cap = bytes;
    }
    if (!b.staged) OCS_CUDA(cudaEventCreateWithFlags(&b.staged, cudaEventDisableTiming));
    if (!b.done) OCS_CUDA(cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming));
    return OCS_OK;
}

void batch_scratch_release(BatchScratch& b)
{
    if (b.host) cudaFreeHost(b.host);
    if (b.dev) cudaFree(b.dev);
    if (b.staged) cudaEventDestroy(b.staged);
    if (b.done) cudaEventDestroy(b.done);
    b = BatchScratch{};
}

int batch_prepare_into(const ocs_request* reqs, int count, BatchScratch& b)
{
    std::vector<ocs_request> copy(reqs, reqs + count);
    BatchPlan bp;
    int rc = batch_build(copy.data(), count, bp, true);
    if (rc) return rc;
    batch_occ_get();
    batch_tiles(bp, kBatchGroupsMin);  // room for the most tiles any tuned length makes
    return batch_scratch_grow(b, batch_bytes(bp.descs.size(), bp.tiles.size()));
}

namespace {

// Stages bp's descriptors and tiles in b and launches the persistent kernel.
int batch_launch(const BatchPlan& bp, cudaStream_t st, BatchScratch& b, bool capturing)
{
    Context& c = ctx();
    const size_t bytes = batch_bytes(bp.descs.size(), bp.tiles.size());
    if (capturing && (b.host_cap < bytes || b.dev_cap < bytes))
        return fail(OCS_ENOMEM, "batch buffers not prepared (call ocs_batch_prepare before each capture)");
    int rc = batch_scratch_grow(b, bytes);
    if (rc) return rc;
    const int occ = batch_occ_get();
    if (!capturing) {
        // the previous batch's descriptors must have left the staging buffer,
        // and its kernel must be done reading the device copy
        OCS_CUDA(cudaEventSynchronize(b.staged));
        OCS_CUDA(cudaStreamWaitEvent(st, b.done, 0));
    }
    const size_t o_tiles = align256(bp.descs.size() * sizeof(ocs::FusedArgs));
    const size_t o_cnt = o_tiles + align256(bp.tiles.size() * sizeof(ocs::BatchTile));
    std::memcpy(b.host, bp.descs.data(), bp.descs.size() * sizeof(ocs::FusedArgs));
    std::memcpy(b.host + o_tiles, bp.tiles.data(), bp.tiles.size() * sizeof(ocs::BatchTile));
    const uint32_t nt = (uint32_t)bp.tiles.size();
    std::memcpy(b.host + o_cnt, &nt, 4);
    std::memset(b.host + o_cnt + 4, 0, 4);  // tile counter starts at zero
    OCS_CUDA(cudaMemcpyAsync(b.dev, b.host, o_cnt + 8, cudaMemcpyHostToDevice, st));
    if (!capturing) OCS_CUDA(cudaEventRecord(b.staged, st));
    auto* d_reqs = reinterpret_cast<const ocs::FusedArgs*>(b.dev);
    auto* d_tiles = reinterpret_cast<const ocs::BatchTile*>(b.dev + o_tiles);
    auto* d_nt = reinterpret_cast<const uint32_t*>(b.dev + o_cnt);
    auto* d_cnt = reinterpret_cast<uint32_t*>(b.dev + o_cnt + 4);
    const int grid = std::max(1, std::min<int>(c.sms * occ, (int)bp.tiles.size()));
    OCS_CUDA(ocs::launch_batch(d_reqs, d_tiles, d_nt, d_cnt, grid, st));
    if (!capturing) OCS_CUDA(cudaEventRecord(b.done, st));
    return OCS_OK;
}

// Times each tile length on this batch (every run writes the same outputs)
// and returns the fastest; the caller's launch then writes them once more.
int batch_tune(BatchPlan& bp, cudaStream_t st, BatchScratch& b, int* best_groups)
{
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t te = cudaEventCreate(&e0);
    if (te == cudaSuccess) te = cudaEventCreate(&e1);
    float best = 1e30f;
    *best_groups = kBatchGroupsDefault;
    int rc = OCS_OK;
    for (int g : kBatchGroups) {
        if (te != cudaSuccess || rc) break;
        batch_tiles(bp, g);
        rc = batch_launch(bp, st, b, false);  // warm-up
        if (!rc) te = cudaEventRecord(e0, st);
        for (int k = 0; k < 2 && !rc && te == cudaSuccess; ++k) rc = batch_launch(bp, st, b, false);
        if (!rc && te == cudaSuccess) te = cudaEventRecord(e1, st);
        if (!rc && te == cudaSuccess) te = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (!rc && te == cudaSuccess) te = cudaEventElapsedTime(&ms, e0, e1);
        if (!rc && te == cudaSuccess && ms < best) {
            best = ms;
            *best_groups = g;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc) return rc;
    if (te != cudaSuccess) return cuda_fail(te, "batch tile timing");
    return OCS_OK;
}

}  // namespace

// Uploads the descriptors of one batch into `b` and launches the persistent
// kernel on `st`.  The scratch is reused only after the previous batch that
// used it has read it (GPU-side wait), so batches on different streams with
// different scratch objects run concurrently.
int batch_enqueue(ocs_request* reqs, int count, cudaStream_t st, BatchScratch& b, bool tune)
{
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    OCS_CUDA(cudaStreamIsCapturing(st, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    BatchPlan bp;
    int rc = batch_build(reqs, count, bp, true);
    if (rc) return rc;
    Context& c = ctx();
    if (!bp.descs.empty()) {
        const auto key = batch_mix_key(bp);
        int groups = kBatchGroupsDefault;
        bool known = false;
        {
            std::lock_guard<std::mutex> lk(c.mu);
            auto it = c.batch_tuned.find(key);
            if (it != c.batch_tuned.end()) {
                groups = it->second;
                known = true;
            }
        }
        // OCS_BATCH_GROUPS=8|16|32|64 fixes the tile length (tests, sweeps)
        if (const char* eg = std::getenv("OCS_BATCH_GROUPS")) {
            for (int g : kBatchGroups)
                if (std::atoi(eg) == g) {
                    groups = g;
                    known = true;
                }
        }
        if (tune && !known && !capturing && !env_is("OCS_AUTOTUNE", "0")) {
            rc = batch_tune(bp, st, b, &groups);
            if (rc) return rc;
            std::lock_guard<std::mutex> lk(c.mu);
            c.batch_tuned[key] = groups;
        }
        batch_tiles(bp, groups);
        rc = batch_launch(bp, st, b, capturing);
        if (rc) return rc;
    }
    for (int i : bp.big) {
        const Request& r = bp.parsed[i];
        reqs[i].status = launch_frames(r, reqs[i].in, reqs[i].n, reqs[i].out, 0, r.geo.frames, st);
    }
    return OCS_OK;
}

int ensure_ready() { return ensure_init(); }
void set_error(int, const std::string& msg) { g_err = msg; }

}  // namespace internal
}  // namespace ocs

extern "C" int ocs_batch_prepare(const ocs_request* reqs, int count)
{
    if (count < 0 || (count > 0 && !reqs)) return fail(OCS_EINVAL, "bad request list");
    int rc = ensure_init();
    if (rc) return rc;
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.batch_mu);
    rc = ocs::internal::batch_prepare_into(reqs, count, c.batch);
    if (rc) return rc;
    if (!c.graph_next) c.graph_next = new ocs::internal::BatchScratch();
    return ocs::internal::batch_prepare_into(reqs, count, *c.graph_next);
}

extern "C" int ocs_batch_device(ocs_request* reqs, int count, void* stream)
{
    if (count < 0 || (count > 0 && !reqs)) return fail(OCS_EINVAL, "bad request list");
    int rc = ensure_init();
    if (rc) return rc;
    const cudaStream_t st = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    OCS_CUDA(cudaStreamIsCapturing(st, &cap));
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.batch_mu);
    if (cap == cudaStreamCaptureStatusNone) return ocs::internal::batch_enqueue(reqs, count, st, c.batch, true);
    if (!c.graph_next)
        return fail(OCS_ENOMEM, "batch buffers not prepared (call ocs_batch_prepare before each capture)");
    rc = ocs::internal::batch_enqueue(reqs, count, st, *c.graph_next);
    if (rc) return rc;
    c.graph_kept.push_back(c.graph_next);
    c.graph_next = nullptr;
    return OCS_OK;
}

namespace ocs {
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace ocs

extern "C" {

int ocs_init(int device)
{
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    return init_locked(c, device);
}

void ocs_shutdown(void)
{
    ocs::internal::noalloc_forget_devices();
    Context& c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    if (!c.ready) return;
    cudaSetDevice(c.device);
    cudaDeviceSynchronize();
    for (auto& kv : c.twiddles) cudaFree(kv.second);
    for (auto& kv : c.windows) cudaFree(kv.second);
    for (auto& kv : c.two_level) cudaFree(kv.second);
    c.twiddles.clear();
    c.windows.clear();
    c.windows_host.clear();
    c.two_level.clear();
    for (Slot* s : c.all_slots) destroy_slot(s);
    c.all_slots.clear();
    c.free_slots.clear();
    c.occupancy.clear();
    ocs::internal::batch_scratch_release(c.batch);
    if (c.graph_next) c.graph_kept.push_back(c.graph_next);
    c.graph_next = nullptr;
    for (auto* g : c.graph_kept) {
        ocs::internal::batch_scratch_release(*g);
        delete g;
    }
    c.graph_kept.clear();
    c.batch_occ = 0;
    if (c.h_err) cudaFreeHost(c.h_err);
    c.h_err = nullptr;
    c.d_err = nullptr;
    if (c.s_setup) cudaStreamDestroy(c.s_setup);
    c.s_setup = nullptr;
    c.ready = false;
}

const char* ocs_last_error(void) { return g_err.c_str(); }

const char* ocs_version(void) { return "occastft_gb300 0.1 (sm_103a)"; }

int ocs_geometry_get(uint64_t n, int exp, float ov, const char* options, ocs_geometry* out)
{
    Request r;
    int rc = prepare(n, exp, ov, options, r);
    if (rc) return rc;
    std::memset(out, 0, sizeof(*out));
    out->qt = r.geo.qt;
    out->hop = r.geo.hop;
    out->ofull = r.geo.ofull;
    out->ohalf = r.geo.ohalf;
    out->n_window = r.geo.n_window;
    out->out_floats = r.geo.out_floats;
    out->frames = r.geo.frames;
    return OCS_OK;
}

int ocs_activate_device(const float* d_in, uint64_t n, int exp, float ov, const char* options, float* d_out,
                        uint64_t out_cap, void* stream)
{
    Request r;
    int rc = prepare(n, exp, ov, options, r);
    if (rc) return rc;
    if (out_cap < r.geo.out_floats) return fail(OCS_ESPACE, "output buffer too small");
    if (!d_in || !d_out) return fail(OCS_EINVAL, "null buffer");
    rc = ensure_init();
    if (rc) return rc;
    // asynchronous: a timed-out earlier tensor-core launch is reported here
    if (r.opt.precision >= 1) {
        rc = take_tc_error();
        if (rc) return rc;
    }
    return launch_frames(r, d_in, n, d_out, 0, r.geo.frames, (cudaStream_t)stream);
}

int ocs_activate(const float* in, uint64_t n, int exp, float ov, const char* options, float* out, uint64_t out_cap,
                 uint64_t* out_len)
{
    Request r;
    int rc = prepare(n, exp, ov, options, r);
    if (rc) return rc;
    if (out_cap < r.geo.out_floats) return fail(OCS_ESPACE, "output buffer too small");
    if (!in || !out) return fail(OCS_EINVAL, "null buffer");
    rc = ensure_init();
    if (rc) return rc;
    Slot* s = acquire_slot(&rc);
    if (!s) return rc;
    const uint64_t N = r.geo.n_window, hop = r.geo.hop, F = r.geo.frames;
    // samples the computed frames read
    const uint64_t need_in = std::min<uint64_t>(n, (F - 1) * hop + N);
    rc = grow(&s->d_in, &s->in_cap, std::max<uint64_t>(need_in, 1));
    if (!rc) rc = grow(&s->d_out, &s->out_cap, std::max<uint64_t>(r.geo.out_floats, 1));
    if (rc) {
        release_slot(s);
        return rc;
    }
    // chunking: ~8 MB of input per chunk (OCS_CHUNK_MB overrides), at most kMaxChunks
    uint64_t chunk_bytes = 8ull << 20;
    if (const char* cm = std::getenv("OCS_CHUNK_MB")) chunk_bytes = (uint64_t)std::min(std::max(1L, std::atol(cm)), 4096L) << 20;
    const uint64_t target = std::max<uint64_t>(1, chunk_bytes / 4 / std::max<uint64_t>(hop, 1));
    uint64_t chunks = std::min<uint64_t>(kMaxChunks, std::max<uint64_t>(1, (F + target - 1) / target));
    const uint64_t per = (F + chunks - 1) / chunks;
    chunks = (F + per - 1) / per;
    // Input prefix copied once chunk ci's host-to-device copy has finished.
    std::vector<uint64_t> in_hi(chunks);
    for (uint64_t ci = 0; ci < chunks; ++ci) {
        const uint64_t f1 = std::min(F, ci * per + per);
        in_hi[ci] = std::min<uint64_t>(need_in, (f1 - 1) * hop + N);
    }
    // In-place use (out overlapping in, e.g. a shared-memory region that
    // holds the signal and receives the result): a device-to-host copy may
    // only overwrite input that has already reached the device, so it also
    // waits for the first host-to-device chunk that covers the input it
    // overlaps.  All input copies are issued first in that case.
    const uintptr_t ib = reinterpret_cast<uintptr_t>(in), ie = ib + need_in * sizeof(float);
    const uintptr_t ob = reinterpret_cast<uintptr_t>(out), oe = ob + r.geo.out_floats * sizeof(float);
    const bool aliased = ob < ie && ib < oe;
    uint64_t copied = 0;
    cudaError_t e = cudaSuccess;
    auto issue_h2d = [&](uint64_t ci) {
        const uint64_t hi = in_hi[ci];
        if (hi > copied) {
            e = cudaMemcpyAsync(s->d_in + copied, in + copied, (hi - copied) * sizeof(float), cudaMemcpyHostToDevice,
                                s->s_h2d);
            copied = hi;
        }
        if (e == cudaSuccess) e = cudaEventRecord(s->ev_in[ci], s->s_h2d);
    };
    if (aliased)
        for (uint64_t ci = 0; ci < chunks && e == cudaSuccess; ++ci) issue_h2d(ci);
    for (uint64_t ci = 0; ci < chunks && e == cudaSuccess; ++ci) {
        const uint64_t f0 = ci * per, f1 = std::min(F, f0 + per);
        if (!aliased) issue_h2d(ci);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s->s_comp, s->ev_in[ci], 0);
        if (e != cudaSuccess) break;
        rc = launch_frames(r, s->d_in, need_in, s->d_out, f0, f1, s->s_comp);
        if (rc) break;
        e = cudaEventRecord(s->ev_comp[ci], s->s_comp);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s->s_d2h, s->ev_comp[ci], 0);
        uint64_t off, cnt;
        out_range(r, f0, f1, &off, &cnt);
        if (e == cudaSuccess && aliased && cnt) {
            const uintptr_t wb = ob + off * sizeof(float), we = wb + cnt * sizeof(float);
            if (wb < ie && ib < we) {
                const uint64_t need = (std::min(we, ie) - ib + sizeof(float) - 1) / sizeof(float);
                uint64_t cj = ci;
                while (cj + 1 < chunks && in_hi[cj] < need) ++cj;
                if (cj > ci) e = cudaStreamWaitEvent(s->s_d2h, s->ev_in[cj], 0);
            }
        }
        if (e == cudaSuccess && cnt)
            e = cudaMemcpyAsync(out + off, s->d_out + off, cnt * sizeof(float), cudaMemcpyDeviceToHost, s->s_d2h);
    }
    cudaError_t e2 = cudaStreamSynchronize(s->s_d2h);
    cudaError_t e3 = cudaStreamSynchronize(s->s_comp);
    release_slot(s);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "ocs_activate");
    if (e2 != cudaSuccess) return cuda_fail(e2, "ocs_activate sync");
    if (e3 != cudaSuccess) return cuda_fail(e3, "ocs_activate sync");
    if (r.opt.precision >= 1) {
        rc = take_tc_error();
        if (rc) return rc;
    }
    if (out_len) *out_len = r.geo.out_floats;
    return OCS_OK;
}

int ocs_plan_tune(uint64_t n, int exp, float ov, const char* options, int* variant)
{
    if (variant) *variant = -1;
    Request r;
    int rc = prepare(n, exp, ov, options, r);
    if (rc) return rc;
    rc = ensure_init();
    if (rc) return rc;
    // windows above the fused kernels and the tensor-core precisions have one form each
    if (ocs::large_supports(r.exp) || r.opt.precision >= 1) return OCS_OK;
    const uint64_t N = r.geo.n_window, hop = r.geo.hop, F = r.geo.frames;
    const uint64_t need_in = std::max<uint64_t>(1, std::min<uint64_t>(n, (F - 1) * hop + N));
    const uint64_t need_out = std::max<uint64_t>(1, r.geo.out_floats);
    Context& c = ctx();
    float* d_in = nullptr;
    float* d_out = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&d_in), need_in * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_out), need_out * sizeof(float));
    if (e == cudaSuccess) e = cudaMemsetAsync(d_in, 0, need_in * sizeof(float), c.s_setup);
    if (e != cudaSuccess) {
        if (d_in) cudaFree(d_in);
        if (d_out) cudaFree(d_out);
        return cuda_fail(e, "plan tuning buffers");
    }
    // the whole request (ocs_activate_device) and one chunk of ocs_activate's
    // copy/compute pipeline: the tuner keys on the frame count's size class
    rc = launch_frames(r, d_in, need_in, d_out, 0, F, c.s_setup);
    const int chosen = g_last_variant;
    if (!rc) {
        const uint64_t target = std::max<uint64_t>(1, (8ull << 20) / 4 / std::max<uint64_t>(hop, 1));
        const uint64_t chunks = std::min<uint64_t>(kMaxChunks, std::max<uint64_t>(1, (F + target - 1) / target));
        const uint64_t per = (F + chunks - 1) / chunks;
        if (per < F) rc = launch_frames(r, d_in, need_in, d_out, 0, per, c.s_setup);
    }
    const cudaError_t es = cudaStreamSynchronize(c.s_setup);
    cudaFree(d_in);
    cudaFree(d_out);
    if (rc) return rc;
    if (es != cudaSuccess) return cuda_fail(es, "plan tuning");
    if (variant) *variant = chosen;
    return OCS_OK;
}

int ocs_window_table(int kind, uint32_t window_size, float sigma, float* out)
{
    if (kind < 1 || kind > 8 || !out || window_size < 2 || (window_size & (window_size - 1)))
        return fail(OCS_EINVAL, "window table: bad arguments");
    const std::vector<float> w = ocs::window_table(kind, (int)window_size, sigma);
    std::memcpy(out, w.data(), sizeof(float) * w.size());
    return OCS_OK;
}

int ocs_host_alloc(void** ptr, size_t bytes)
{
    cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return fail(OCS_ENOMEM, std::string("pinned allocation failed: ") + cudaGetErrorString(e));
    }
    return OCS_OK;
}

int ocs_host_free(void* ptr)
{
    OCS_CUDA(cudaFreeHost(ptr));
    return OCS_OK;
}

int ocs_host_register(void* ptr, size_t bytes)
{
    if (!ptr || !bytes) return fail(OCS_EINVAL, "host register: empty range");
    int rc = ensure_init();
    if (rc) return rc;
    OCS_CUDA(cudaHostRegister(ptr, bytes, cudaHostRegisterPortable));
    return OCS_OK;
}

int ocs_host_unregister(void* ptr)
{
    OCS_CUDA(cudaHostUnregister(ptr));
    return OCS_OK;
}

// ---------------------------------------------------------------- stage hooks
int ocs_stage_overlap(const float* d_origin, uint32_t ofull, uint32_t full_size, uint32_t exp, uint32_t hop,
                      float* d_real, void* stream)
{
    if (exp < 6 || exp > 30 || !d_origin || !d_real || full_size == 0) return fail(OCS_EINVAL, "Overlap: bad arguments");
    int rc = ensure_init();
    if (rc) return rc;
    OCS_CUDA(ocs::launch_overlap(d_origin, ofull, full_size, exp, hop, d_real, (cudaStream_t)stream));
    return OCS_OK;
}

int ocs_stage_window(int kind, float* d_data, uint32_t ofull, uint32_t window_size, float sigma, void* stream)
{
    if (kind < 1 || kind > 8 || !d_data || window_size < 64 || (window_size & (window_size - 1)))
        return fail(OCS_EINVAL, "window: bad arguments");
    int exp = 0;
    while ((1u << exp) < window_size) ++exp;
    if (exp > ocs::kLargeMaxExp) return fail(OCS_EINVAL, "window: size above 2^30");
    int rc = ensure_init();
    if (rc) return rc;
    const float* w = nullptr;
    rc = get_window(kind, exp, sigma, false, &w);
    if (rc) return rc;
    OCS_CUDA(ocs::launch_apply_window(d_data, w, ofull, window_size, (cudaStream_t)stream));
    return OCS_OK;
}

int ocs_stage_remove_dc(float* d_data, uint32_t qt, uint32_t ofull, uint32_t window_size, void* stream)
{
    (void)qt;
    if (!d_data || window_size < 64 || (window_size & (window_size - 1))) return fail(OCS_EINVAL, "RemoveDC: bad arguments");
    int rc = ensure_init();
    if (rc) return rc;
    OCS_CUDA(ocs::launch_remove_dc(d_data, ofull, window_size, (cudaStream_t)stream));
    return OCS_OK;
}

int ocs_stage_fft(float* d_real, float* d_imag, uint32_t ohalf, uint32_t exp, void* stream)
{
    if (exp < 6) return fail(OCS_EINVAL, "Operation not supported");
    if (exp > (uint32_t)ocs::kLargeMaxExp) return fail(OCS_EINVAL, "Operation not supported: window sizes above 2^30");
    if (!d_real || !d_imag) return fail(OCS_EINVAL, "EXP: null buffer");
    int rc = ensure_init();
    if (rc) return rc;
    if (ocs::large_supports((int)exp)) {
        // EXPC above the one-launch sizes: the four-step FFT of every frame of
        // the real plane, no window, full N-bin spectra into both planes.  The
        // frames are chunked and each chunk's column pass reads its frames
        // before its row pass writes them, so the transform runs in place.
        const uint64_t N = 1ull << exp;
        const uint64_t frames = 2ull * ohalf / N;
        return launch_large_core((int)exp, ocs::OUT_PLANES, d_real, 2ull * ohalf, N, nullptr, 0, 0, 0, d_real, d_imag,
                                 0, frames, (cudaStream_t)stream);
    }
    const float2* tw = nullptr;
    rc = get_twiddles((int)exp, false, &tw);
    if (rc) return rc;
    const float* half = nullptr;  // all-1/2 table: the untangle's scale, no window
    rc = get_window(ocs::WIN_NONE, (int)exp, -1.0f, true, &half);
    if (rc) return rc;
    const uint64_t N = 1ull << exp;
    ocs::FusedArgs a{};
    a.x = d_real;
    a.n = 2ull * ohalf;
    a.hop = N;
    a.frames = 2ull * ohalf / N;
    a.win = half;
    a.tw = tw;
    a.out = d_real;
    a.out_im = d_imag;
    a.vec2 = (reinterpret_cast<uintptr_t>(d_real) & 7u) == 0;
    if (a.frames == 0) return OCS_OK;
    OCS_CUDA(ocs::launch_fused((int)exp, ocs::OUT_PLANES, false, a,
                               grid_size((int)exp, ocs::OUT_PLANES, VAR_DIRECT, a.frames), (cudaStream_t)stream));
    return OCS_OK;
}

int ocs_stage_half_complex(float* d_out, const float* d_real, const float* d_imag, uint32_t ohalf, uint32_t exp,
                           void* stream)
{
    (void)exp;
    if (!d_out || !d_real || !d_imag) return fail(OCS_EINVAL, "HalfComplex: null buffer");
    int rc = ensure_init();
    if (rc) return rc;
    OCS_CUDA(ocs::launch_half_complex(d_out, d_real, d_imag, ohalf, (cudaStream_t)stream));
    return OCS_OK;
}

int ocs_stage_to_power(float* d_out, const float* d_real, const float* d_imag, uint32_t ofull, void* stream)
{
    if (!d_out || !d_real || !d_imag) return fail(OCS_EINVAL, "ToPower: null buffer");
    int rc = ensure_init();
    if (rc) return rc;
    OCS_CUDA(ocs::launch_to_power(d_out, d_real, d_imag, ofull, (cudaStream_t)stream));
    return OCS_OK;
}

}  // extern "C"
