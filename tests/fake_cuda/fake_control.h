// TEST INFRASTRUCTURE ONLY: knobs and counters of the host-only CUDA stand-in
// (cuda_runtime.h in this folder) and of its stand-in batch launch.
#pragma once
#include <atomic>
#include <cstdint>

namespace fake {

// a cudaMemcpyAsync from or to this address fails (cudaErrorInvalidValue)
extern std::atomic<const void*> fail_copy_ptr;
// stream creations left before cudaStreamCreateWithFlags fails (< 0: never)
extern std::atomic<int> stream_fail_after;
// how long one batch launch occupies its stream, microseconds
extern std::atomic<int> kernel_us;
// live device allocations and streams (leak checks)
extern std::atomic<long> live_allocs;
extern std::atomic<long> live_streams;
// batch launches issued, and the largest request count of one launch
extern std::atomic<long> launches;
extern std::atomic<long> max_launch_requests;

// The stand-in "STFT" the fake batch launch writes: a deterministic function
// of the request's input, so every output can be checked on the host.
inline float expected(const float* in, uint64_t n, int exp, uint64_t k)
{
    return in[k % n] * 0.5f + (float)exp;
}

}  // namespace fake
