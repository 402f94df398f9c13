// TEST INFRASTRUCTURE ONLY: knobs and counters of the host-only CUDA stand-in
// (cuda_runtime.h in this folder) and of its stand-in kernels.
#pragma once
#include <atomic>
#include <cstdint>
#include <functional>

#include "cuda_runtime.h"

namespace fake {

// a cudaMemcpyAsync from or to this address fails (cudaErrorInvalidValue)
extern std::atomic<const void*> fail_copy_ptr;
// creations left before cudaStreamCreateWithFlags / cudaEventCreate* fail (< 0: never)
extern std::atomic<int> stream_fail_after;
extern std::atomic<int> event_fail_after;
// likewise for cudaHostAlloc and for host-to-device copies
extern std::atomic<int> host_alloc_fail_after;
extern std::atomic<int> h2d_fail_after;
// the stream cudaStreamIsCapturing reports as capturing (null: none)
extern std::atomic<cudaStream_t> capturing;
// source addresses of the host-to-device copies issued on `capturing`
void captured_sources(std::function<void(const void*, size_t)> fn);
// each unit of stream work first sleeps up to this many microseconds (random)
extern std::atomic<int> jitter_us;
// each host-to-device copy first sleeps this long: copies that a later
// device-to-host copy must wait for then finish late
extern std::atomic<int> h2d_delay_us;
// how long one stand-in batch launch occupies its stream, microseconds
extern std::atomic<int> kernel_us;
// live device allocations, pinned host allocations, streams and events
extern std::atomic<long> live_allocs;
extern std::atomic<long> live_host_allocs;
extern std::atomic<long> live_streams;
extern std::atomic<long> live_events;
// batch launches issued, and the largest request count of one launch
extern std::atomic<long> launches;
extern std::atomic<long> max_launch_requests;
// stand-in kernel launches (ocs_api tests)
extern std::atomic<long> kernel_launches;

// queues work on a stream (the stand-in kernels use this)
void enqueue(cudaStream_t st, std::function<void()> fn);

// The stand-in "STFT" of the request server test: a deterministic function of
// the request's input, so every output can be checked on the host.
inline float expected(const float* in, uint64_t n, int exp, uint64_t k)
{
    return in[k % n] * 0.5f + (float)exp;
}

}  // namespace fake
