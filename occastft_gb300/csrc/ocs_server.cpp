// Continuous-batching STFT request server.
//
// Replaces the reference's one-request-at-a-time WebSocket callback
// (StandAlone/cross_gpgpu/GLOBAL/RunnerCommon.cpp:69-134), which parses a
// request, runs ActivateSTFT to completion (allocating and freeing device
// memory every time) and only then reads the next message.  Here:
//   * requests are queued as they arrive (ocs_server_submit returns at once);
//   * a worker thread admits queued requests into one of S in-flight slots
//     as soon as a slot is free and the device pool has room for their input
//     and output (admission by free HBM, first come first served);
//   * an admitted group is copied host->device, run as ONE persistent batch
//     launch (ocs_batch kernel, mixed window sizes / overlaps / outputs) and
//     copied back, all on the slot's stream, so groups in different slots
//     overlap their copies and compute on the device;
//   * a host callback on the slot's stream stamps completion times; latency
//     is submit-to-completion and reported as p50 / p99 / p999.
#include "ocs_host.h"
#include "ocs_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;
using ocs::internal::BatchScratch;

double now_ms()
{
    return std::chrono::duration<double, std::milli>(Clock::now().time_since_epoch()).count();
}

// first-fit allocator over the device pool, 256-byte granules
class PoolAlloc {
public:
    void reset(size_t cap)
    {
        free_.clear();
        free_[0] = cap;
        cap_ = cap;
        used_ = 0;
    }
    bool alloc(size_t bytes, size_t* off)
    {
        bytes = (bytes + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, start = it->first + bytes;
                free_.erase(it);
                if (rest) free_[start] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes)
    {
        bytes = (bytes + 255) & ~(size_t)255;
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t capacity() const { return cap_; }
    size_t used() const { return used_; }

private:
    std::map<size_t, size_t> free_;
    size_t cap_ = 0, used_ = 0;
};

struct Job {
    uint64_t ticket = 0;
    const float* in = nullptr;
    uint64_t n = 0;
    int exp = 0;
    float ov = 0.0f;
    std::string options;
    float* out = nullptr;
    uint64_t out_floats = 0;
    size_t in_off = 0, out_off = 0, in_bytes = 0, out_bytes = 0;
    double t_submit = 0.0, t_done = 0.0;
    int status = -1;
    bool done = false;
    bool cancelled = false;
};

struct Server;

struct Slot {
    Server* srv = nullptr;
    cudaStream_t st = nullptr;
    BatchScratch scratch;
    std::vector<std::shared_ptr<Job>> jobs;
    bool busy = false;
    std::atomic<bool> finished{false};
    double t_done = 0.0;
};

struct Server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Job>> pending;
    std::map<uint64_t, std::shared_ptr<Job>> jobs;
    std::vector<std::unique_ptr<Slot>> slots;
    PoolAlloc pool;
    char* d_pool = nullptr;
    int max_batch = 256;
    uint64_t next_ticket = 1;
    bool running = false;
    std::thread worker;
    int device = 0;
    // statistics
    double t_start = 0.0;
    uint64_t completed = 0, failed = 0, rejected = 0, samples = 0, batches = 0;
    std::vector<double> lat_ms;  // ring of the most recent kLatencyWindow latencies
    size_t lat_next = 0;
    double lat_max = 0.0;
};

constexpr size_t kLatencyWindow = size_t(1) << 20;

// The running server.  Calls take a reference under g_ptr_mu, so a stop
// that runs meanwhile never frees a server another call is still using;
// g_life_mu keeps starts and stops one at a time.  The holder is never
// destroyed: a server still running at process exit is left alone rather
// than destroyed with its worker thread attached.
std::shared_ptr<Server>& g_srv = *new std::shared_ptr<Server>();
std::mutex g_ptr_mu;
std::mutex g_life_mu;

std::shared_ptr<Server> current()
{
    std::lock_guard<std::mutex> g(g_ptr_mu);
    return g_srv;
}

// Frees the slots' streams and scratch and the device pool (no worker running).
void release_resources(Server& S)
{
    for (auto& s : S.slots) {
        if (!s->st) continue;
        cudaStreamSynchronize(s->st);
        ocs::internal::batch_scratch_release(s->scratch);
        cudaStreamDestroy(s->st);
        s->st = nullptr;
    }
    if (S.d_pool) cudaFree(S.d_pool);
    S.d_pool = nullptr;
}

int err(int code, const std::string& m)
{
    ocs::internal::set_error(code, m);
    return code;
}

void CUDART_CB on_slot_done(void* p)
{
    Slot* s = static_cast<Slot*>(p);
    s->t_done = now_ms();
    s->finished.store(true);
    std::lock_guard<std::mutex> lk(s->srv->mu);
    s->srv->cv_work.notify_one();
}

// called with the lock held
void reap(Server& S)
{
    for (auto& sp : S.slots) {
        Slot& s = *sp;
        if (!s.busy || !s.finished.load()) continue;
        for (auto& j : s.jobs) {
            S.pool.release(j->in_off, j->in_bytes);
            S.pool.release(j->out_off, j->out_bytes);
            j->t_done = s.t_done;
            j->done = true;
            if (j->status == OCS_OK) {
                ++S.completed;
                S.samples += j->n;
                const double ms = j->t_done - j->t_submit;
                if (S.lat_ms.size() < kLatencyWindow) {
                    S.lat_ms.push_back(ms);
                } else {
                    S.lat_ms[S.lat_next] = ms;
                    S.lat_next = (S.lat_next + 1) % kLatencyWindow;
                }
                S.lat_max = std::max(S.lat_max, ms);
            } else {
                ++S.failed;
            }
        }
        s.jobs.clear();
        s.busy = false;
        s.finished.store(false);
        S.cv_done.notify_all();
    }
}

// A request whose copy to or from the device cannot be issued fails with
// OCS_ECUDA; the copy's error is cleared so the batch launch does not take it
// for its own.
void issue(Server& S, Slot& s)
{
    std::vector<ocs_request> reqs;
    std::vector<size_t> job_of;  // s.jobs index of each request
    reqs.reserve(s.jobs.size());
    job_of.reserve(s.jobs.size());
    for (size_t i = 0; i < s.jobs.size(); ++i) {
        Job& j = *s.jobs[i];
        float* din = reinterpret_cast<float*>(S.d_pool + j.in_off);
        float* dout = reinterpret_cast<float*>(S.d_pool + j.out_off);
        if (cudaMemcpyAsync(din, j.in, j.n * 4, cudaMemcpyHostToDevice, s.st) != cudaSuccess) {
            cudaGetLastError();
            j.status = OCS_ECUDA;
            continue;
        }
        reqs.push_back(ocs_request{din, j.n, j.exp, j.ov, j.options.c_str(), dout, j.out_floats, -1, 0});
        job_of.push_back(i);
    }
    const int rc =
        reqs.empty() ? OCS_OK : ocs::internal::batch_enqueue(reqs.data(), (int)reqs.size(), s.st, s.scratch);
    for (size_t k = 0; k < reqs.size(); ++k) {
        Job& j = *s.jobs[job_of[k]];
        j.status = rc ? rc : reqs[k].status;
        if (j.status == OCS_OK &&
            cudaMemcpyAsync(j.out, S.d_pool + j.out_off, j.out_floats * 4, cudaMemcpyDeviceToHost, s.st) !=
                cudaSuccess) {
            cudaGetLastError();
            j.status = OCS_ECUDA;
        }
    }
    if (cudaLaunchHostFunc(s.st, on_slot_done, &s) != cudaSuccess) {
        cudaStreamSynchronize(s.st);
        on_slot_done(&s);
    }
}

void worker_main(Server* Sp)
{
    Server& S = *Sp;
    cudaSetDevice(S.device);
    std::unique_lock<std::mutex> lk(S.mu);
    while (S.running || !S.pending.empty() ||
           std::any_of(S.slots.begin(), S.slots.end(), [](const std::unique_ptr<Slot>& s) { return s->busy; })) {
        reap(S);
        bool issued = false;
        for (auto& sp : S.slots) {
            Slot& s = *sp;
            if (s.busy || S.pending.empty()) continue;
            while (!S.pending.empty() && (int)s.jobs.size() < S.max_batch) {
                std::shared_ptr<Job> j = S.pending.front();
                if (j->cancelled) {
                    S.pending.pop_front();
                    continue;
                }
                size_t a, b;
                if (!S.pool.alloc(j->in_bytes, &a)) break;
                if (!S.pool.alloc(j->out_bytes, &b)) {
                    S.pool.release(a, j->in_bytes);
                    break;
                }
                j->in_off = a;
                j->out_off = b;
                s.jobs.push_back(j);
                S.pending.pop_front();
            }
            if (s.jobs.empty()) break;  // the pool is full: wait for a slot to finish
            s.busy = true;
            ++S.batches;
            lk.unlock();
            issue(S, s);
            lk.lock();
            issued = true;
        }
        if (!issued) S.cv_work.wait_for(lk, std::chrono::microseconds(200));
    }
}

}  // namespace

extern "C" {

int ocs_server_start(const ocs_server_config* cfg)
{
    std::lock_guard<std::mutex> g(g_life_mu);
    if (current()) return err(OCS_EINVAL, "server already running");
    int rc = ocs::internal::ensure_ready();
    if (rc) return rc;
    auto S = std::make_shared<Server>();
    cudaGetDevice(&S->device);
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    size_t pool = cfg && cfg->pool_bytes ? (size_t)cfg->pool_bytes : fr / 2;
    if (pool > fr) return err(OCS_ENOMEM, "pool larger than free device memory");
    if (cudaMalloc((void**)&S->d_pool, pool) != cudaSuccess) {
        cudaGetLastError();
        return err(OCS_ENOMEM, "cannot allocate the request pool");
    }
    S->pool.reset(pool);
    S->max_batch = cfg && cfg->max_batch > 0 ? cfg->max_batch : 256;
    const int nslots = cfg && cfg->slots > 0 ? cfg->slots : 3;
    for (int i = 0; i < nslots; ++i) {
        auto s = std::make_unique<Slot>();
        s->srv = S.get();
        if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess) {
            release_resources(*S);
            return err(OCS_ECUDA, "stream creation failed");
        }
        S->slots.push_back(std::move(s));
    }
    S->running = true;
    S->t_start = now_ms();
    S->worker = std::thread(worker_main, S.get());
    std::lock_guard<std::mutex> p(g_ptr_mu);
    g_srv = S;
    return OCS_OK;
}

int ocs_server_submit(const float* in, uint64_t n, int window_size_exp, float overlap_ratio, const char* options,
                      float* out, uint64_t out_cap, uint64_t* ticket)
{
    const std::shared_ptr<Server> S = current();
    if (!S) return err(OCS_EINVAL, "server not running");
    if (!in || !out || !ticket) return err(OCS_EINVAL, "null argument");
    ocs_geometry g;
    int rc = ocs_geometry_get(n, window_size_exp, overlap_ratio, options, &g);
    if (rc) return rc;
    if (out_cap < g.out_floats) return err(OCS_ESPACE, "output buffer too small");
    auto j = std::make_shared<Job>();
    j->in = in;
    j->n = n;
    j->exp = window_size_exp;
    j->ov = overlap_ratio;
    j->options = options ? options : "";
    j->out = out;
    j->out_floats = g.out_floats;
    j->in_bytes = n * 4;
    j->out_bytes = g.out_floats * 4;
    if (((j->in_bytes + 255) & ~(size_t)255) + ((j->out_bytes + 255) & ~(size_t)255) > S->pool.capacity()) {
        std::lock_guard<std::mutex> lk(S->mu);
        ++S->rejected;
        return err(OCS_ENOMEM, "request larger than the server's device pool");
    }
    std::lock_guard<std::mutex> lk(S->mu);
    if (!S->running) return err(OCS_EINVAL, "server stopping");
    j->ticket = S->next_ticket++;
    j->t_submit = now_ms();
    S->jobs[j->ticket] = j;
    S->pending.push_back(j);
    *ticket = j->ticket;
    S->cv_work.notify_one();
    return OCS_OK;
}

int ocs_server_wait(uint64_t ticket, int timeout_ms, int* status)
{
    const std::shared_ptr<Server> S = current();
    if (!S) return err(OCS_EINVAL, "server not running");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->jobs.find(ticket);
    if (it == S->jobs.end()) return err(OCS_EINVAL, "unknown ticket");
    std::shared_ptr<Job> j = it->second;
    const bool ok = S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 1 << 30 : timeout_ms),
                                        [&] { return j->done; });
    if (!ok) return err(OCS_ETIMEDOUT, "request not finished within the timeout");
    if (status) *status = j->status;
    S->jobs.erase(ticket);
    return OCS_OK;
}

int ocs_server_cancel(uint64_t ticket)
{
    const std::shared_ptr<Server> S = current();
    if (!S) return err(OCS_EINVAL, "server not running");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->jobs.find(ticket);
    if (it == S->jobs.end()) return err(OCS_EINVAL, "unknown ticket");
    auto& j = it->second;
    if (j->done) return err(OCS_EINVAL, "request already finished");
    auto p = std::find(S->pending.begin(), S->pending.end(), j);
    if (p == S->pending.end()) return err(OCS_EINVAL, "request already on the device");
    S->pending.erase(p);
    S->jobs.erase(it);
    return OCS_OK;
}

int ocs_server_get_stats(ocs_server_stats* out)
{
    const std::shared_ptr<Server> S = current();
    if (!S || !out) return err(OCS_EINVAL, "server not running");
    std::vector<double> l;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        std::memset(out, 0, sizeof(*out));
        out->completed = S->completed;
        out->failed = S->failed;
        out->rejected = S->rejected;
        out->pending = S->pending.size();
        out->batches = S->batches;
        out->samples = S->samples;
        out->elapsed_ms = now_ms() - S->t_start;
        out->pool_bytes = S->pool.capacity();
        out->pool_used = S->pool.used();
        out->max_ms = S->lat_max;
        l = S->lat_ms;
    }
    if (!l.empty()) {
        // sorted outside the lock, so the worker is not held up
        std::sort(l.begin(), l.end());
        auto q = [&](double p) { return l[std::min(l.size() - 1, (size_t)(p * (l.size() - 1) + 0.5))]; };
        out->p50_ms = q(0.50);
        out->p99_ms = q(0.99);
        out->p999_ms = q(0.999);
    }
    return OCS_OK;
}

int ocs_server_reset_stats(void)
{
    const std::shared_ptr<Server> S = current();
    if (!S) return err(OCS_EINVAL, "server not running");
    std::lock_guard<std::mutex> lk(S->mu);
    S->completed = S->failed = S->rejected = S->samples = S->batches = 0;
    S->lat_ms.clear();
    S->lat_next = 0;
    S->lat_max = 0.0;
    S->t_start = now_ms();
    return OCS_OK;
}

int ocs_server_stop(void)
{
    std::lock_guard<std::mutex> g(g_life_mu);
    const std::shared_ptr<Server> S = current();
    if (!S) return err(OCS_EINVAL, "server not running");
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->running = false;
        S->cv_work.notify_all();
    }
    S->worker.join();
    release_resources(*S);
    std::lock_guard<std::mutex> p(g_ptr_mu);
    g_srv.reset();
    return OCS_OK;
}

}  // extern "C"
