// TEST INFRASTRUCTURE ONLY: the host-only CUDA stand-in and the library
// internals the request server links against (batch launch, error text,
// geometry), for compiling occastft_gb300/csrc/ocs_server.cpp without a GPU.
// Geometry and option parsing are the library's own (ocs_host.cpp, linked
// beside this file); only the device work is replaced.
#include "cuda_runtime.h"
#include "fake_control.h"
#include "ocs_host.h"
#include "ocs_internal.h"

#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace fake {
std::atomic<const void*> fail_copy_ptr{nullptr};
std::atomic<int> stream_fail_after{-1};
std::atomic<int> kernel_us{200};
std::atomic<long> live_allocs{0};
std::atomic<long> live_streams{0};
std::atomic<long> launches{0};
std::atomic<long> max_launch_requests{0};
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
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [&] { return quit || !q.empty(); });
            if (q.empty()) return;
            std::function<void()> f = std::move(q.front());
            q.pop_front();
            busy = true;
            lk.unlock();
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

namespace {
thread_local cudaError_t t_last = cudaSuccess;
thread_local std::string t_err;

cudaError_t set_last(cudaError_t e)
{
    t_last = e;
    return e;
}
}  // namespace

cudaError_t cudaGetDevice(int* device)
{
    *device = 0;
    return cudaSuccess;
}
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaMemGetInfo(size_t* free_bytes, size_t* total_bytes)
{
    *free_bytes = size_t(1) << 30;
    *total_bytes = size_t(2) << 30;
    return cudaSuccess;
}
cudaError_t cudaMalloc(void** p, size_t bytes)
{
    *p = std::aligned_alloc(256, (bytes + 255) & ~size_t(255));
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
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* st, unsigned)
{
    int left = fake::stream_fail_after.load();
    if (left == 0) return set_last(cudaErrorMemoryAllocation);
    if (left > 0) fake::stream_fail_after.store(left - 1);
    *st = new FakeStream();
    ++fake::live_streams;
    return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t st)
{
    if (!st) return set_last(cudaErrorInvalidValue);
    delete st;
    --fake::live_streams;
    return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t st)
{
    if (!st) return set_last(cudaErrorInvalidValue);
    st->sync();
    return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t bytes, cudaMemcpyKind, cudaStream_t st)
{
    const void* bad = fake::fail_copy_ptr.load();
    if (bad && (bad == src || bad == dst)) return set_last(cudaErrorInvalidValue);
    st->push([=] { std::memcpy(dst, src, bytes); });
    return cudaSuccess;
}
cudaError_t cudaLaunchHostFunc(cudaStream_t st, cudaHostFn_t fn, void* arg)
{
    st->push([=] { fn(arg); });
    return cudaSuccess;
}
cudaError_t cudaGetLastError(void)
{
    const cudaError_t e = t_last;
    t_last = cudaSuccess;
    return e;
}
const char* cudaGetErrorString(cudaError_t e) { return e ? "fake CUDA error" : "no error"; }

namespace ocs {
void set_last_error(const std::string& msg) { t_err = msg; }

namespace internal {

// The batch launch: validates each request as the library does and queues one
// unit of stream work that writes fake::expected() into every output.
int batch_enqueue(ocs_request* reqs, int count, cudaStream_t st, BatchScratch&)
{
    struct Item {
        const float* in;
        uint64_t n;
        int exp;
        float* out;
        uint64_t out_floats;
    };
    std::vector<Item> items;
    for (int i = 0; i < count; ++i) {
        ocs_request& q = reqs[i];
        Options o;
        Geometry g;
        std::string st_msg = parse_options(q.options, o);
        q.status = st_msg == "OK" ? OCS_OK : OCS_EPIPELINE;
        if (q.status == OCS_OK && make_geometry(q.n, q.window_size_exp, q.overlap_ratio, o, g) != "OK")
            q.status = OCS_EINVAL;
        if (q.status == OCS_OK && q.out_cap < g.out_floats) q.status = OCS_ESPACE;
        if (q.status == OCS_OK) items.push_back(Item{q.in, q.n, q.window_size_exp, q.out, g.out_floats});
    }
    ++fake::launches;
    long prev = fake::max_launch_requests.load();
    while (prev < count && !fake::max_launch_requests.compare_exchange_weak(prev, count)) {
    }
    const int us = fake::kernel_us.load();
    st->push([items, us] {
        std::this_thread::sleep_for(std::chrono::microseconds(us));
        for (const Item& it : items)
            for (uint64_t k = 0; k < it.out_floats; ++k) it.out[k] = fake::expected(it.in, it.n, it.exp, k);
    });
    return OCS_OK;
}

void batch_scratch_release(BatchScratch& b) { b = BatchScratch{}; }
int ensure_ready() { return OCS_OK; }
void set_error(int, const std::string& msg) { t_err = msg; }

}  // namespace internal
}  // namespace ocs

extern "C" int ocs_geometry_get(uint64_t n, int exp, float ov, const char* options, ocs_geometry* out)
{
    ocs::Options o;
    ocs::Geometry g;
    std::string s = ocs::parse_options(options, o);
    if (s != "OK") {
        t_err = s;
        return OCS_EPIPELINE;
    }
    s = ocs::make_geometry(n, exp, ov, o, g);
    if (s != "OK") {
        t_err = s;
        return OCS_EINVAL;
    }
    std::memset(out, 0, sizeof(*out));
    out->qt = g.qt;
    out->hop = g.hop;
    out->ofull = g.ofull;
    out->ohalf = g.ohalf;
    out->n_window = g.n_window;
    out->out_floats = g.out_floats;
    out->frames = g.frames;
    return OCS_OK;
}

extern "C" const char* ocs_last_error(void) { return t_err.c_str(); }
