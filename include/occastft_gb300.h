/*
 * occastft_gb300 — C ABI of the GB300 (sm_103a) STFT runner.
 *
 * This library is the drop-in for OCCAstft's CUDA runner: the calls below
 * replace, one for one, what the reference's runner contract exposes
 * (StandAlone/cross_gpgpu/GLOBAL/RunnerInterface.hpp) and what its CUDA
 * vendor implementation does (StandAlone/cross_gpgpu/CUDA/src/CudaImpl.cpp,
 * StandAlone/cross_gpgpu/CUDA/src/functionImpl.cpp).  Signatures use plain
 * pointers and sizes only; `stream` arguments are cudaStream_t handles passed
 * as void* (NULL = the legacy default stream).
 *
 * Option strings follow the reference grammar (RunnerCommon.cpp:166-253):
 *   --hanning_window --hamming_window --blackman_window --nuttall_window
 *   --blackman_nuttall_window --blackman_harris_window --flattop_window
 *   --gaussian_window=<sigma><<sigma   --remove_dc   --half_complex_return
 * with the reference's precedence (first window in that order wins) and its
 * sigma parsing.  Two additive flags select a layout the reference lacks:
 *   --layout=dense   N/2+1 bins per frame (power: qt*(N/2+1) floats,
 *                    half-complex: qt*(N/2+1) interleaved complex)
 *   --serial_power   power = sqrt(2)*|Re X|, the value the reference's
 *                    Serial/OpenMP runners return (default: |X|, the value
 *                    of the reference's toPower kernel)
 *
 * All entry points are thread-safe.  Status codes: OCS_OK or one of OCS_E*;
 * ocs_last_error() then holds the message (for pipeline failures it is the
 * reference's own status string, e.g. "Operation not supported" or
 * "--gaussian_window").
 */
#ifndef OCCASTFT_GB300_H
#define OCCASTFT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OCS_OK 0
#define OCS_EINVAL 1    /* unsupported size/overlap/option ("Operation not supported") */
#define OCS_EPIPELINE 2 /* the option string fails the reference's parsing ("--gaussian_window") */
#define OCS_ENOMEM 3    /* device or pinned-host allocation failed / admission refused */
#define OCS_ECUDA 4     /* a CUDA call failed */
#define OCS_ESPACE 5    /* the output buffer is smaller than the layout needs */
#define OCS_ETIMEDOUT 6 /* a bounded device wait expired */

/* Frame geometry of one request (all values as the reference computes them). */
typedef struct ocs_geometry {
    uint32_t qt;          /* frame count, toQuot() */
    uint32_t hop;         /* OMove */
    uint32_t ofull;       /* OFullSize = qt * N */
    uint32_t ohalf;       /* OHalfSize = OFullSize / 2 */
    uint32_t n_window;    /* N = 1 << windowSizeEXP */
    uint32_t reserved;
    uint64_t out_floats;  /* floats the selected layout writes */
    uint64_t frames;      /* frames the device computes (compat half-complex needs only ceil(qt/2)) */
} ocs_geometry;

/* Runner::InitEnv + Runner::BuildKernel (CudaImpl.cpp:285-407): select the
 * device, size launch grids.  Calling it is optional (the first request
 * initialises the current device). */
int ocs_init(int device);

/* Runner::UnInit: release every cached plan, buffer and stream. */
void ocs_shutdown(void);

/* Message of the last failing call on this thread ("" when none). */
const char* ocs_last_error(void);

const char* ocs_version(void);

/* Sizes of a request: toQuot (RunnerInterface.hpp:26-35) and the sizing block
 * of ActivateSTFT (CudaImpl.cpp:416-421), plus the output length the options
 * select. */
int ocs_geometry_get(uint64_t n, int window_size_exp, float overlap_ratio, const char* options,
                     ocs_geometry* out);

/* Runner::ActivateSTFT (RunnerInterface.hpp:124-128; CUDA version
 * CudaImpl.cpp:410-510): host signal in, host result out, synchronous.
 * out must hold geometry.out_floats floats; *out_len receives that count.
 * Host buffers from ocs_host_alloc give the fastest copies.  out may overlap
 * in (the result written over the signal): each part of the result is copied
 * back only after the input it overwrites has reached the device. */
int ocs_activate(const float* in, uint64_t n, int window_size_exp, float overlap_ratio, const char* options,
                 float* out, uint64_t out_cap, uint64_t* out_len);

/* The device half of ActivateSTFT: runnerFunction::Default_Pipeline
 * (RunnerCommon.cpp:184-316) on device-resident buffers, fused into one
 * kernel launch on `stream`, asynchronous.  With --precision=tc-fp16 a wait
 * inside the tensor-core kernel that gives up (after about a second) is
 * reported as OCS_ETIMEDOUT by ocs_activate at once and, since this call
 * does not synchronise, by the next tensor-core call of this function. */
int ocs_activate_device(const float* d_in, uint64_t n, int window_size_exp, float overlap_ratio,
                        const char* options, float* d_out, uint64_t out_cap, void* stream);

/* Plan tuning ahead of the first request (new; the reference has no
 * counterpart).  Times the kernel variants that apply to requests of this
 * shape (window size, output kind and layout, and the size class of the
 * frame count, for the whole request and for one chunk of ocs_activate's
 * copy/compute pipeline) on scratch buffers of that size, and keeps the
 * fastest, as the first call of that shape would.  *variant (may be NULL)
 * receives the variant the whole request runs: 0 one frame per FFT, 1 the
 * same with staged I/O, 2 two frames per FFT, 3 lanes per frame, 4 two
 * frames per FFT on packed FP32x2; -1 where the shape has one form (windows
 * above 2^15, tensor-core precisions).  With OCS_AUTOTUNE=0 nothing is timed
 * and the default variant is reported.  Synchronous. */
int ocs_plan_tune(uint64_t n, int window_size_exp, float overlap_ratio, const char* options, int* variant);

/* The window coefficients the runner applies (host computation, no device
 * needed): the reference's formulas (OKL/kernel.okl:33-127) evaluated with
 * the same float/double roundings as its Serial runner, so they match that
 * runner bit for bit on the same host.  kind as in ocs_stage_window;
 * out receives window_size floats. */
int ocs_window_table(int kind, uint32_t window_size, float sigma, float* out);

/* Pinned host memory for inputs/outputs of ocs_activate. */
int ocs_host_alloc(void** ptr, size_t bytes);
int ocs_host_free(void* ptr);

/* Pins an existing host range (a mapped shared-memory payload, say) for the
 * copies of ocs_activate, and releases it again.  No counterpart in the
 * reference, whose runners copy such payloads into new vectors first. */
int ocs_host_register(void* ptr, size_t bytes);
int ocs_host_unregister(void* ptr);

/* ---- uneven batches: many requests, one persistent launch ---- */

/* One request of a batch.  For ocs_batch_device `in` and `out` are device
 * pointers.  `status` is written by the call: OCS_OK or the request's error. */
typedef struct ocs_request {
    const float* in;
    uint64_t n;
    int window_size_exp;
    float overlap_ratio;
    const char* options;
    float* out;
    uint64_t out_cap; /* floats */
    int status;
    int reserved;
} ocs_request;

/* Builds the plans (twiddle and window tables) these requests need and grows
 * the batch's descriptor buffers, so that a following ocs_batch_device over
 * requests of the same shapes allocates nothing and can be captured into a
 * CUDA graph.  It also sets aside descriptor buffers for the next captured
 * ocs_batch_device: call it once before each capture.  Replaces nothing in
 * the reference (its runner handles one request at a time,
 * RunnerCommon.cpp:69-134). */
int ocs_batch_prepare(const ocs_request* reqs, int count);

/* Runs all valid requests (windows 2^6..2^13) as tiles of one persistent
 * kernel launch on `stream` (requests with larger windows get their own
 * fused launch on the same stream).  Asynchronous.  Returns OCS_OK when the
 * launch was issued; per-request problems land in reqs[i].status.
 * Under stream capture it uses the buffers the last ocs_batch_prepare set
 * aside (OCS_ENOMEM if there are none, or they are too small) and keeps them
 * until ocs_shutdown, so the graph replays its own requests whatever batches
 * run after the capture.  Replays of one graph must not overlap each other on
 * the GPU (they share those buffers); replays and other batches may.
 * The first call outside capture for a new mix of window sizes and batch
 * size times the tile lengths (8 .. 64 frame groups per tile) on these
 * requests, running the batch about a dozen times, and waits for that; the
 * outputs are the same for every length.  OCS_AUTOTUNE=0 skips this. */
int ocs_batch_device(ocs_request* reqs, int count, void* stream);

/* Same as ocs_batch_device, for callers that must not allocate GPU memory
 * (an application that owns the whole device through its own allocator, or
 * a process that must never block on or fail in cudaMalloc once running).
 * No counterpart in the reference.  It allocates nothing: its scratch and
 * tables live in a fixed 1 MiB device array inside the library, held on every
 * GPU that loads the library until the process exits.  Limits (rejected with
 * OCS_ENOMEM and a message): at most 256 requests per call, windows 2^6..2^13,
 * distinct window tables of one call within the array's window region.
 * Requests with larger windows, or with a --precision=tc-* option (the
 * tensor-core forms need tables the array has no room for), get status
 * OCS_EINVAL.  When a call fails with OCS_ENOMEM, every request it accepted
 * gets that status too (nothing was launched).  The first call on a device
 * (with that device current) sets the array up and synchronizes `stream`
 * once; CUDA loads the library's device code lazily, so that is also when
 * the array takes its device memory: call once with count = 0 (set-up only)
 * before an allocator of your own reserves the device.  ocs_shutdown forgets
 * the set-up, so a call after a device reset sets it up again.
 * Calls cannot be captured into a CUDA graph (OCS_EINVAL):
 * their descriptors go through a host staging buffer that every call
 * rewrites.  All calls share the array: calls whose work overlaps on the GPU
 * race, so order them on one stream or with events. */
int ocs_batch_device_noalloc(ocs_request* reqs, int count, void* stream);

/* ---- serving: a continuous-batching request server ----
 * Replaces the reference's one-request-at-a-time WebSocket callback
 * (GLOBAL/RunnerCommon.cpp:69-134).  Requests (host buffers) queue on submit;
 * a worker admits them into in-flight slots as slots and device-pool memory
 * free up, runs each admitted group as one persistent batch launch between
 * its host->device and device->host copies, and overlaps the slots on the
 * device.  Latency is submit-to-completion. */
typedef struct ocs_server_config {
    uint64_t pool_bytes; /* device pool for in-flight requests; 0 = half of free memory */
    int max_batch;       /* requests per launch; 0 = 256 */
    int slots;           /* groups in flight; 0 = 3 */
} ocs_server_config;

typedef struct ocs_server_stats {
    uint64_t completed, failed, rejected, pending, batches, samples;
    double elapsed_ms; /* since start or the last reset */
    /* p50/p99/p999 over the most recent 2^20 completed requests; max over
     * all completed since start or the last reset */
    double p50_ms, p99_ms, p999_ms, max_ms;
    uint64_t pool_bytes, pool_used;
} ocs_server_stats;

int ocs_server_start(const ocs_server_config* cfg);
/* Queues one request; in/out are host buffers that must stay valid until
 * ocs_server_wait returns (pinned buffers copy fastest).  Fails with
 * OCS_ENOMEM when the request alone exceeds the device pool.  A request
 * whose copy to or from the device cannot be issued finishes with status
 * OCS_ECUDA.  The server calls may run on any threads, including a stop
 * while other threads submit or wait. */
int ocs_server_submit(const float* in, uint64_t n, int window_size_exp, float overlap_ratio, const char* options,
                      float* out, uint64_t out_cap, uint64_t* ticket);
/* Waits up to timeout_ms (< 0: no limit) for a request; *status is its result. */
int ocs_server_wait(uint64_t ticket, int timeout_ms, int* status);
/* Withdraws a request that has not been admitted yet (a client that left). */
int ocs_server_cancel(uint64_t ticket);
int ocs_server_get_stats(ocs_server_stats* out);
int ocs_server_reset_stats(void);
/* Finishes every queued request, then stops. */
int ocs_server_stop(void);

/* ---- per-stage hooks: runnerFunction::* (RunnerInterface.hpp:38-76) on
 * device buffers laid out as the reference's [qt][N] planes. ---- */

/* runnerFunction::Overlap (CUDA/src/functionImpl.cpp:15-55) */
int ocs_stage_overlap(const float* d_origin, uint32_t ofull, uint32_t full_size, uint32_t window_size_exp,
                      uint32_t hop, float* d_real, void* stream);

/* runnerFunction::Hanning .. FlatTop, Gaussian (functionImpl.cpp:58-270);
 * kind: 1 Hanning, 2 Hamming, 3 Blackman, 4 Nuttall, 5 Blackman-Nuttall,
 * 6 Blackman-Harris, 7 FlatTop, 8 Gaussian(sigma) */
int ocs_stage_window(int kind, float* d_data, uint32_t ofull, uint32_t window_size, float sigma, void* stream);

/* runnerFunction::RemoveDC (functionImpl.cpp:276-305) */
int ocs_stage_remove_dc(float* d_data, uint32_t qt, uint32_t ofull, uint32_t window_size, void* stream);

/* runnerFunction::EXP6..EXP11 and EXPC (functionImpl.cpp:346-609): FFT of
 * each frame of the real plane (imaginary input ignored, as the reference's
 * first stage does), full N-bin spectra written back into d_real/d_imag. */
int ocs_stage_fft(float* d_real, float* d_imag, uint32_t ohalf, uint32_t window_size_exp, void* stream);

/* runnerFunction::HalfComplex (functionImpl.cpp:612-647) */
int ocs_stage_half_complex(float* d_out, const float* d_real, const float* d_imag, uint32_t ohalf,
                           uint32_t window_size_exp, void* stream);

/* runnerFunction::ToPower (functionImpl.cpp:650-683) */
int ocs_stage_to_power(float* d_out, const float* d_real, const float* d_imag, uint32_t ofull, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* OCCASTFT_GB300_H */
