// TEST INFRASTRUCTURE ONLY: the host-only CUDA stand-in declared in
// cuda_runtime.h.  Streams are FIFO worker threads, events record a
// generation on the host and complete it in stream order, and
// cudaStreamWaitEvent makes a stream's worker wait for that generation, so
// work on different streams is ordered exactly as far as the events order
// it.  An optional random delay before each unit of stream work shakes out
// orderings that the events do not enforce.
#include "cuda_runtime.h"
#include "fake_control.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <utility>
#include <vector>

namespace fake {
std::atomic<const void*> fail_copy_ptr{nullptr};
std::atomic<int> stream_fail_after{-1};
std::atomic<int> event_fail_after{-1};
std::atomic<int> host_alloc_fail_after{-1};
std::atomic<int> h2d_fail_after{-1};
std::atomic<cudaStream_t> capturing{nullptr};
std::atomic<int> jitter_us{0};
std::atomic<int> h2d_delay_us{0};
std::atomic<int> kernel_us{200};
std::atomic<long> live_allocs{0};
std::atomic<long> live_host_allocs{0};
std::atomic<long> live_streams{0};
std::atomic<long> live_events{0};
std::atomic<long> launches{0};
std::atomic<long> max_launch_requests{0};
std::atomic<long> kernel_launches{0};

namespace {
std::mutex g_cap_mu;
std::vector<std::pair<const void*, size_t>> g_captured;

// creations left before a failure; false when this creation fails
bool take(std::atomic<int>& left)
{
    int v = left.load();
    while (v > 0 && !left.compare_exchange_weak(v, v - 1)) {
    }
    return v != 0;
}
}  // namespace

void captured_sources(std::function<void(const void*, size_t)> fn)
{
    std::lock_guard<std::mutex> lk(g_cap_mu);
    for (const auto& c : g_captured) fn(c.first, c.second);
}
}  // namespace fake

// One stream: a worker thread running queued work in submission order.
struct FakeStream {
    std::mutex mu;
    std::condition_variable cv, cv_idle;
    std::deque<std::function<void()>> q;
    bool busy = false;
    bool quit = false;
    std::thread th;  // last: starts after the members above exist

    FakeStream() : th([this] { run(); }) {}
    ~FakeStream()
    {
        {
            std::lock_guard<std::mutex> lk(mu);
            quit = true;
        }
        cv.notify_one();
        th.join();
    }
    void run()
    {
        std::mt19937 rng((unsigned)std::hash<std::thread::id>()(std::this_thread::get_id()));
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [&] { return quit || !q.empty(); });
            if (q.empty()) return;
            std::function<void()> f = std::move(q.front());
            q.pop_front();
            busy = true;
            lk.unlock();
            const int j = fake::jitter_us.load();
            if (j > 0) std::this_thread::sleep_for(std::chrono::microseconds(rng() % (unsigned)(j + 1)));
            f();
            lk.lock();
            busy = false;
            if (q.empty()) cv_idle.notify_all();
        }
    }
    void push(std::function<void()> f)
    {
        {
            std::lock_guard<std::mutex> lk(mu);
            q.push_back(std::move(f));
        }
        cv.notify_one();
    }
    void sync()
    {
        std::unique_lock<std::mutex> lk(mu);
        cv_idle.wait(lk, [&] { return q.empty() && !busy; });
    }
};

struct FakeEvent {
    std::mutex mu;
    std::condition_variable cv;
    uint64_t recorded = 0, completed = 0;
    double t_ms = 0.0;
};

namespace {
thread_local cudaError_t t_last = cudaSuccess;

cudaError_t set_last(cudaError_t e)
{
    t_last = e;
    return e;
}

// the legacy default stream (null handle)
FakeStream* stream_of(cudaStream_t st)
{
    static FakeStream* legacy = new FakeStream();  // never destroyed
    return st ? st : legacy;
}

double now_ms()
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

void fake::enqueue(cudaStream_t st, std::function<void()> fn) { stream_of(st)->push(std::move(fn)); }

cudaError_t cudaGetDevice(int* device)
{
    *device = 0;
    return cudaSuccess;
}
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int)
{
    std::memset(p, 0, sizeof(*p));
    std::strcpy(p->name, "host stand-in");
    p->major = 10;
    p->minor = 3;
    p->multiProcessorCount = 8;
    return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize(void)
{
    stream_of(nullptr)->sync();
    return cudaSuccess;
}
cudaError_t cudaMemGetInfo(size_t* free_bytes, size_t* total_bytes)
{
    *free_bytes = size_t(1) << 30;
    *total_bytes = size_t(2) << 30;
    return cudaSuccess;
}
cudaError_t cudaMalloc(void** p, size_t bytes)
{
    *p = std::aligned_alloc(256, std::max<size_t>(256, (bytes + 255) & ~size_t(255)));
    if (!*p) return set_last(cudaErrorMemoryAllocation);
    ++fake::live_allocs;
    return cudaSuccess;
}
cudaError_t cudaFree(void* p)
{
    if (p) {
        std::free(p);
        --fake::live_allocs;
    }
    return cudaSuccess;
}
cudaError_t cudaMallocAsync(void** p, size_t bytes, cudaStream_t) { return cudaMalloc(p, bytes); }
cudaError_t cudaFreeAsync(void* p, cudaStream_t st)
{
    // freed once the stream's earlier work has run
    stream_of(st)->push([p] { cudaFree(p); });
    return cudaSuccess;
}
cudaError_t cudaHostAlloc(void** p, size_t bytes, unsigned)
{
    if (!fake::take(fake::host_alloc_fail_after)) return set_last(cudaErrorMemoryAllocation);
    *p = std::aligned_alloc(256, std::max<size_t>(256, (bytes + 255) & ~size_t(255)));
    if (!*p) return set_last(cudaErrorMemoryAllocation);
    ++fake::live_host_allocs;
    return cudaSuccess;
}
cudaError_t cudaFreeHost(void* p)
{
    if (p) {
        std::free(p);
        --fake::live_host_allocs;
    }
    return cudaSuccess;
}
cudaError_t cudaHostGetDevicePointer(void** d, void* h, unsigned)
{
    *d = h;
    return cudaSuccess;
}
cudaError_t cudaHostRegister(void*, size_t, unsigned) { return cudaSuccess; }
cudaError_t cudaHostUnregister(void*) { return cudaSuccess; }

cudaError_t cudaStreamCreateWithFlags(cudaStream_t* st, unsigned)
{
    if (!fake::take(fake::stream_fail_after)) return set_last(cudaErrorMemoryAllocation);
    *st = new FakeStream();
    ++fake::live_streams;
    return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t st)
{
    if (!st) return set_last(cudaErrorInvalidValue);
    st->sync();
    delete st;
    --fake::live_streams;
    return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t st)
{
    stream_of(st)->sync();
    return cudaSuccess;
}
cudaError_t cudaStreamIsCapturing(cudaStream_t st, cudaStreamCaptureStatus* status)
{
    *status = (st && st == fake::capturing.load()) ? cudaStreamCaptureStatusActive : cudaStreamCaptureStatusNone;
    return cudaSuccess;
}
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* ev, unsigned)
{
    if (!fake::take(fake::event_fail_after)) return set_last(cudaErrorMemoryAllocation);
    *ev = new FakeEvent();
    ++fake::live_events;
    return cudaSuccess;
}
cudaError_t cudaEventCreate(cudaEvent_t* ev) { return cudaEventCreateWithFlags(ev, 0); }
cudaError_t cudaEventDestroy(cudaEvent_t ev)
{
    if (!ev) return set_last(cudaErrorInvalidValue);
    { std::lock_guard<std::mutex> lk(ev->mu); }  // a completing record has left it
    delete ev;
    --fake::live_events;
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t ev, cudaStream_t st)
{
    uint64_t gen;
    {
        std::lock_guard<std::mutex> lk(ev->mu);
        gen = ++ev->recorded;
    }
    stream_of(st)->push([ev, gen] {
        // signalled under the lock: a host thread that sees the completion
        // may destroy the event at once, as it may a CUDA event
        std::lock_guard<std::mutex> lk(ev->mu);
        ev->completed = std::max(ev->completed, gen);
        ev->t_ms = now_ms();
        ev->cv.notify_all();
    });
    return cudaSuccess;
}
cudaError_t cudaStreamWaitEvent(cudaStream_t st, cudaEvent_t ev, unsigned)
{
    uint64_t gen;
    {
        std::lock_guard<std::mutex> lk(ev->mu);
        gen = ev->recorded;
    }
    if (gen == 0) return cudaSuccess;  // never recorded: nothing to wait for
    stream_of(st)->push([ev, gen] {
        std::unique_lock<std::mutex> lk(ev->mu);
        ev->cv.wait(lk, [&] { return ev->completed >= gen; });
    });
    return cudaSuccess;
}
cudaError_t cudaEventSynchronize(cudaEvent_t ev)
{
    std::unique_lock<std::mutex> lk(ev->mu);
    const uint64_t gen = ev->recorded;
    ev->cv.wait(lk, [&] { return ev->completed >= gen; });
    return cudaSuccess;
}
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t start, cudaEvent_t end)
{
    std::lock_guard<std::mutex> a(start->mu);
    std::lock_guard<std::mutex> b(end->mu);
    *ms = (float)std::max(0.0, end->t_ms - start->t_ms);
    return cudaSuccess;
}
cudaError_t cudaMemsetAsync(void* dst, int value, size_t bytes, cudaStream_t st)
{
    stream_of(st)->push([dst, value, bytes] { std::memset(dst, value, bytes); });
    return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st)
{
    const void* bad = fake::fail_copy_ptr.load();
    if (bad && (bad == src || bad == dst)) return set_last(cudaErrorInvalidValue);
    if (kind == cudaMemcpyHostToDevice && !fake::take(fake::h2d_fail_after)) return set_last(cudaErrorInvalidValue);
    if (st && st == fake::capturing.load() && kind == cudaMemcpyHostToDevice) {
        std::lock_guard<std::mutex> lk(fake::g_cap_mu);
        fake::g_captured.emplace_back(src, bytes);
    }
    const int delay = kind == cudaMemcpyHostToDevice ? fake::h2d_delay_us.load() : 0;
    stream_of(st)->push([=] {
        if (delay > 0) std::this_thread::sleep_for(std::chrono::microseconds(delay));
        std::memcpy(dst, src, bytes);
    });
    return cudaSuccess;
}
cudaError_t cudaLaunchHostFunc(cudaStream_t st, cudaHostFn_t fn, void* arg)
{
    stream_of(st)->push([=] { fn(arg); });
    return cudaSuccess;
}
cudaError_t cudaGetLastError(void)
{
    const cudaError_t e = t_last;
    t_last = cudaSuccess;
    return e;
}
const char* cudaGetErrorString(cudaError_t e) { return e ? "stand-in CUDA error" : "no error"; }
