// TEST INFRASTRUCTURE ONLY: drives the C ABI's host logic
// (occastft_gb300/csrc/ocs_api.cpp compiled unchanged) against the host-only
// CUDA stand-in and stand-in kernels in this folder.  Each check prints
// "ok <name>"; the first failure prints "FAIL <name>: <why>" and exits 1.
//
//   setup_fail    a set-up whose pinned error word cannot be allocated
//                 releases its stream, and a later ocs_init starts over
//   table_fail    a window table whose upload cannot be issued is freed
//   slot_fail     a request slot whose streams cannot all be created is
//                 released again (no stream or event left behind)
//   tune_fail     a kernel-variant timing whose events cannot be created
//                 fails the request and leaves no event behind
//   activate      ocs_activate on random sizes, overlaps and layouts, with
//                 several copy/compute chunks and random delays on every
//                 stream: the result equals the stand-in kernels' rule, with
//                 separate buffers and with the result written over the
//                 signal (same start, output after input, input after output)
//   concurrent    four threads calling ocs_activate at once, tuning on:
//                 every result correct (run under ThreadSanitizer, this also
//                 checks the shared plan, window, tuning and slot state)
//   batch         ocs_batch_device over mixed requests, windows 2^6 .. 2^16
//   capture_tune  ocs_activate_device on a capturing stream never times
//                 kernel variants (no event is made, nothing synchronises);
//                 it runs before any check that tunes other keys
//   capture       a captured batch keeps its own descriptor buffers: a later
//                 batch does not touch them; a capture without a preceding
//                 ocs_batch_prepare is refused
//   shutdown      ocs_shutdown releases every allocation, stream and event
//
// With arguments it runs one half of the tuning-cache check instead, each in
// a fresh process: "tune-cache-write <file>" tunes one request with
// OCS_TUNE_CACHE=<file>; "tune-cache-read <file>" runs the same request where
// no event can be created, so it succeeds only on the cached choice.
#include "../../include/occastft_gb300.h"
#include "fake_control.h"
#include "fake_expect.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>

namespace {

void check(bool ok, const char* name, const std::string& why)
{
    if (ok) return;
    std::printf("FAIL %s: %s (last error: %s)\n", name, why.c_str(), ocs_last_error());
    std::fflush(stdout);
    std::exit(1);
}

std::vector<float> expected_out(const float* x, uint64_t n, int exp, float ov, const std::string& opts)
{
    std::vector<float> v = fake::expected_out(x, n, exp, ov, opts);
    check(!v.empty(), "expected_out", "geometry");
    return v;
}

using fake::make_signal;

const char* kOpts[] = {"--hanning_window", "--hamming_window --half_complex_return", "--blackman_window --layout=dense",
                       "--hanning_window --half_complex_return --layout=dense", "--remove_dc --serial_power"};

void setup_fail()
{
    const char* name = "setup_fail";
    fake::host_alloc_fail_after = 0;
    const int rc = ocs_init(0);
    fake::host_alloc_fail_after = -1;
    check(rc == OCS_ECUDA, name, "rc " + std::to_string(rc));
    check(fake::live_streams.load() == 0 && fake::live_host_allocs.load() == 0, name, "set-up objects left behind");
    check(ocs_init(0) == OCS_OK, name, "a second ocs_init");
    check(fake::live_streams.load() == 1 && fake::live_host_allocs.load() == 1, name, "set-up objects");
    std::printf("ok %s\n", name);
}

void table_fail()
{
    const char* name = "table_fail";
    // the device entry point makes no input copies: the first host-to-device
    // copy is the new window table's upload
    std::vector<float> x = make_signal(20000, 3);
    float* d_in = nullptr;
    float* d_out = nullptr;
    ocs_geometry g;
    const char* opts = "--blackman_harris_window";
    check(ocs_geometry_get(x.size(), 7, 0.5f, opts, &g) == OCS_OK, name, "geometry");
    check(cudaMalloc(&d_in, x.size() * 4) == cudaSuccess && cudaMalloc(&d_out, g.out_floats * 4) == cudaSuccess, name,
          "alloc");
    std::memcpy(d_in, x.data(), x.size() * 4);
    const long allocs0 = fake::live_allocs.load();
    fake::h2d_fail_after = 0;
    const int rc = ocs_activate_device(d_in, x.size(), 7, 0.5f, opts, d_out, g.out_floats, nullptr);
    fake::h2d_fail_after = -1;
    check(rc == OCS_ECUDA, name, "rc " + std::to_string(rc));
    // the twiddle tables of window 2^7 stay (they were built); the window table must not
    const long allocs1 = fake::live_allocs.load();
    check(allocs1 - allocs0 == 2, name, "allocations after the failed upload: " + std::to_string(allocs1 - allocs0));
    check(ocs_activate_device(d_in, x.size(), 7, 0.5f, opts, d_out, g.out_floats, nullptr) == OCS_OK, name, "retry");
    cudaStreamSynchronize(nullptr);
    check(std::memcmp(d_out, expected_out(x.data(), x.size(), 7, 0.5f, opts).data(), g.out_floats * 4) == 0, name,
          "result after the retry");
    cudaFree(d_in);
    cudaFree(d_out);
    std::printf("ok %s\n", name);
}

void slot_fail()
{
    const char* name = "slot_fail";
    const long streams0 = fake::live_streams.load(), events0 = fake::live_events.load();
    fake::stream_fail_after = 1;  // the slot's second stream cannot be created
    std::vector<float> x = make_signal(5000, 1), out(1 << 16);
    uint64_t len = 0;
    const int rc = ocs_activate(x.data(), x.size(), 8, 0.5f, "", out.data(), out.size(), &len);
    fake::stream_fail_after = -1;
    check(rc == OCS_ECUDA, name, "rc " + std::to_string(rc));
    check(fake::live_streams.load() == streams0, name, "streams left behind");
    check(fake::live_events.load() == events0, name, "events left behind");
    std::printf("ok %s\n", name);
}

void tune_fail()
{
    const char* name = "tune_fail";
    setenv("OCS_AUTOTUNE", "1", 1);
    std::vector<float> x = make_signal(300000, 2);
    ocs_geometry g;
    check(ocs_geometry_get(x.size(), 11, 0.5f, "", &g) == OCS_OK, name, "geometry");
    std::vector<float> out(g.out_floats);
    uint64_t len = 0;
    // a first request makes the slot (its 32 events); the window and size class here are new,
    // so the next request times the kernel variants first
    check(ocs_activate(x.data(), 1000, 7, 0.5f, "", out.data(), out.size(), &len) == OCS_OK, name, "warm");
    const long events0 = fake::live_events.load();
    fake::event_fail_after = 1;  // the timing's second event cannot be created
    const int rc = ocs_activate(x.data(), x.size(), 11, 0.5f, "", out.data(), out.size(), &len);
    fake::event_fail_after = -1;
    check(rc == OCS_ECUDA, name, "rc " + std::to_string(rc));
    check(fake::live_events.load() == events0, name, "timing events left behind");
    // and the same request succeeds, timed, once events can be made again
    check(ocs_activate(x.data(), x.size(), 11, 0.5f, "", out.data(), out.size(), &len) == OCS_OK, name, "retry");
    check(std::memcmp(out.data(), expected_out(x.data(), x.size(), 11, 0.5f, "").data(), out.size() * 4) == 0, name,
          "tuned result");
    setenv("OCS_AUTOTUNE", "0", 1);
    std::printf("ok %s\n", name);
}

void activate()
{
    const char* name = "activate";
    fake::jitter_us = 150;
    std::mt19937_64 rng(12345);
    const int exps[] = {6, 7, 8, 9, 10, 12, 13, 16};
    const float ovs[] = {0.0f, 0.25f, 0.5f, 0.75f, 0.3f};
    int cases = 0, multi = 0, large_small_budget = 0;
    for (int c = 0; c < 40; ++c) {
        const int exp = exps[rng() % 8];
        const float ov = ovs[rng() % 5];
        const std::string opts = kOpts[rng() % 5];
        // mostly a few copy/compute chunks (about 2M samples each), sometimes one
        const uint64_t n = (c % 4 == 0) ? 1 + rng() % 300000 : 2200000 + rng() % 2600000;
        const int alias = c % 4;  // 0 separate, 1 same start, 2 output after input, 3 input after output
        ocs_geometry g;
        if (ocs_geometry_get(n, exp, ov, opts.c_str(), &g) != OCS_OK) continue;
        if (g.out_floats > (64u << 20)) continue;
        std::vector<float> x = make_signal(n, 100 + c);
        const std::vector<float> want = expected_out(x.data(), n, exp, ov, opts);
        const uint64_t d = 1 + rng() % 4096;
        const uint64_t off_in = alias == 3 ? d : 0, off_out = alias == 2 ? d : 0;
        std::vector<float> buf, sep;
        float* in;
        float* out;
        if (alias == 0) {
            buf = x;
            sep.assign(g.out_floats, -7.0f);
            in = buf.data();
            out = sep.data();
        } else {
            buf.assign(std::max(n + off_in, g.out_floats + off_out), -7.0f);
            std::memcpy(buf.data() + off_in, x.data(), n * 4);
            in = buf.data() + off_in;
            out = buf.data() + off_out;
        }
        // every other request with slow input copies: a result copy that did
        // not wait for the input it overwrites would then overtake it
        fake::h2d_delay_us = (c / 4) % 2 ? 4000 : 0;
        // windows above 2^15 run in launch pairs over frame ranges sized by a
        // scratch budget: a 1 MB budget makes many of them per chunk
        const bool small_budget = c % 3 != 2;
        if (small_budget) setenv("OCS_LARGE_SCRATCH_MB", "1", 1);
        uint64_t len = 0;
        const int rc = ocs_activate(in, n, exp, ov, opts.c_str(), out, g.out_floats, &len);
        unsetenv("OCS_LARGE_SCRATCH_MB");
        fake::h2d_delay_us = 0;
        const std::string tag = "case " + std::to_string(c) + " exp " + std::to_string(exp) + " ov " +
                                std::to_string(ov) + " n " + std::to_string(n) + " alias " + std::to_string(alias) +
                                " '" + opts + "'";
        check(rc == OCS_OK && len == g.out_floats, name, tag + ": rc " + std::to_string(rc));
        check(std::memcmp(out, want.data(), g.out_floats * 4) == 0, name, tag + ": result differs");
        ++cases;
        multi += n > 2200000;
        large_small_budget += exp >= 16 && small_budget;
    }
    fake::jitter_us = 0;
    check(cases >= 30 && multi >= 15 && large_small_budget >= 2, name, "too few cases ran");
    std::printf("ok %s (%d requests, %d with several chunks, %d large windows on a 1 MB scratch budget)\n", name,
                cases, multi, large_small_budget);
}

void concurrent()
{
    const char* name = "concurrent";
    setenv("OCS_AUTOTUNE", "1", 1);
    fake::jitter_us = 50;
    std::vector<std::thread> th;
    std::vector<int> bad(4, 0);
    for (int t = 0; t < 4; ++t) {
        th.emplace_back([t, &bad] {
            std::mt19937 rng(900 + t);
            const int exps[] = {6, 7, 8, 9, 10, 11, 12, 14};
            for (int i = 0; i < 6; ++i) {
                const int exp = exps[rng() % 8];
                const float ov = (rng() % 2) ? 0.5f : 0.75f;
                const std::string opts = kOpts[rng() % 5];
                const uint64_t n = 1000 + rng() % 400000;
                std::vector<float> x = make_signal(n, 7000 + 10 * t + i);
                ocs_geometry g;
                if (ocs_geometry_get(n, exp, ov, opts.c_str(), &g) != OCS_OK) continue;
                std::vector<float> out(g.out_floats, -7.0f);
                uint64_t len = 0;
                if (ocs_activate(x.data(), n, exp, ov, opts.c_str(), out.data(), out.size(), &len) != OCS_OK ||
                    std::memcmp(out.data(), expected_out(x.data(), n, exp, ov, opts).data(), out.size() * 4) != 0)
                    ++bad[t];
            }
        });
    }
    for (auto& t : th) t.join();
    fake::jitter_us = 0;
    setenv("OCS_AUTOTUNE", "0", 1);
    for (int t = 0; t < 4; ++t) check(bad[t] == 0, name, "thread " + std::to_string(t) + " got wrong results");
    std::printf("ok %s\n", name);
}

struct DevReq {
    float* in = nullptr;
    float* out = nullptr;
    std::vector<float> x;
    int exp = 0;
    float ov = 0;
    std::string opts;
    uint64_t out_floats = 0;
};

std::vector<DevReq> make_batch(uint32_t seed, int count)
{
    std::mt19937 rng(seed);
    const int exps[] = {6, 7, 8, 9, 10, 11, 12, 13, 14, 16};
    const float ovs[] = {0.0f, 0.25f, 0.5f, 0.75f, 0.3f};
    std::vector<DevReq> v(count);
    for (int i = 0; i < count; ++i) {
        DevReq& r = v[i];
        r.exp = exps[rng() % 10];
        r.ov = ovs[rng() % 5];
        r.opts = kOpts[rng() % 5];
        const uint64_t N = 1ull << r.exp;
        r.x = make_signal(N / 2 + rng() % (6 * N), seed * 1000 + i);
        ocs_geometry g;
        check(ocs_geometry_get(r.x.size(), r.exp, r.ov, r.opts.c_str(), &g) == OCS_OK, "make_batch", "geometry");
        r.out_floats = g.out_floats;
        check(cudaMalloc(&r.in, r.x.size() * 4) == cudaSuccess && cudaMalloc(&r.out, g.out_floats * 4) == cudaSuccess,
              "make_batch", "alloc");
        std::memcpy(r.in, r.x.data(), r.x.size() * 4);
        for (uint64_t k = 0; k < g.out_floats; ++k) r.out[k] = -7.0f;
    }
    return v;
}

std::vector<ocs_request> requests(const std::vector<DevReq>& v)
{
    std::vector<ocs_request> q(v.size());
    for (size_t i = 0; i < v.size(); ++i)
        q[i] = ocs_request{v[i].in, v[i].x.size(), v[i].exp, v[i].ov, v[i].opts.c_str(), v[i].out, v[i].out_floats, -1, 0};
    return q;
}

void check_batch(const std::vector<DevReq>& v, const std::vector<ocs_request>& q, const char* name)
{
    for (size_t i = 0; i < v.size(); ++i) {
        check(q[i].status == OCS_OK, name, "status " + std::to_string(q[i].status));
        const std::vector<float> want = expected_out(v[i].x.data(), v[i].x.size(), v[i].exp, v[i].ov, v[i].opts);
        check(std::memcmp(v[i].out, want.data(), v[i].out_floats * 4) == 0, name,
              "request " + std::to_string(i) + " exp " + std::to_string(v[i].exp) + " '" + v[i].opts + "' differs");
    }
}

void free_batch(std::vector<DevReq>& v)
{
    for (auto& r : v) {
        cudaFree(r.in);
        cudaFree(r.out);
    }
}

void batch()
{
    const char* name = "batch";
    fake::jitter_us = 100;
    cudaStream_t st;
    check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess, name, "stream");
    for (int round = 0; round < 3; ++round) {
        std::vector<DevReq> v = make_batch(7 + round, 40);
        std::vector<ocs_request> q = requests(v);
        check(ocs_batch_device(q.data(), (int)q.size(), st) == OCS_OK, name, "launch");
        cudaStreamSynchronize(st);
        check_batch(v, q, name);
        free_batch(v);
    }
    cudaStreamDestroy(st);
    fake::jitter_us = 0;
    std::printf("ok %s\n", name);
}

void batch_tune()
{
    const char* name = "batch_tune";
    setenv("OCS_AUTOTUNE", "1", 1);
    cudaStream_t st;
    check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess, name, "stream");
    std::vector<DevReq> v = make_batch(31, 60);
    std::vector<ocs_request> q = requests(v);
    // a new mix: every tile length is timed (4 lengths x 3 launches), then the batch runs once more
    long l0 = fake::launches.load();
    check(ocs_batch_device(q.data(), (int)q.size(), st) == OCS_OK, name, "tuned launch");
    cudaStreamSynchronize(st);
    check(fake::launches.load() - l0 == 13, name, "launches " + std::to_string(fake::launches.load() - l0));
    check_batch(v, q, name);
    // the same mix again: the kept choice, one launch
    l0 = fake::launches.load();
    check(ocs_batch_device(q.data(), (int)q.size(), st) == OCS_OK, name, "second launch");
    cudaStreamSynchronize(st);
    check(fake::launches.load() - l0 == 1, name, "second call tuned again");
    check_batch(v, q, name);
    // a fixed length: no timing for a new mix either
    free_batch(v);
    v = make_batch(32, 20);
    q = requests(v);
    setenv("OCS_BATCH_GROUPS", "32", 1);
    l0 = fake::launches.load();
    check(ocs_batch_device(q.data(), (int)q.size(), st) == OCS_OK, name, "fixed length");
    cudaStreamSynchronize(st);
    check(fake::launches.load() - l0 == 1, name, "fixed length timed");
    check_batch(v, q, name);
    unsetenv("OCS_BATCH_GROUPS");
    free_batch(v);
    cudaStreamDestroy(st);
    setenv("OCS_AUTOTUNE", "0", 1);
    std::printf("ok %s\n", name);
}

void capture()
{
    const char* name = "capture";
    cudaStream_t st, cap;
    check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) == cudaSuccess,
          name, "streams");
    std::vector<DevReq> a = make_batch(21, 30), b = make_batch(22, 45);
    std::vector<ocs_request> qa = requests(a), qb = requests(b);
    check(ocs_batch_prepare(qa.data(), (int)qa.size()) == OCS_OK, name, "prepare");
    fake::capturing = cap;
    check(ocs_batch_device(qa.data(), (int)qa.size(), cap) == OCS_OK, name, "captured launch");
    // a second capture without a prepare in between has no buffers of its own
    check(ocs_batch_device(qa.data(), (int)qa.size(), cap) == OCS_ENOMEM, name, "second capture must be refused");
    fake::capturing = nullptr;
    cudaStreamSynchronize(cap);
    check_batch(a, qa, name);
    // the descriptor bytes the captured upload reads
    std::vector<std::pair<const void*, std::vector<char>>> snap;
    fake::captured_sources([&](const void* p, size_t n) {
        snap.emplace_back(p, std::vector<char>((const char*)p, (const char*)p + n));
    });
    check(!snap.empty(), name, "no captured upload seen");
    // later batches, eager, larger: they must not write into those bytes
    for (int i = 0; i < 2; ++i) {
        check(ocs_batch_device(qb.data(), (int)qb.size(), st) == OCS_OK, name, "eager launch");
        cudaStreamSynchronize(st);
    }
    check_batch(b, qb, name);
    for (const auto& s : snap)
        check(std::memcmp(s.first, s.second.data(), s.second.size()) == 0, name,
              "a later batch rewrote the captured descriptors");
    free_batch(a);
    free_batch(b);
    cudaStreamDestroy(st);
    cudaStreamDestroy(cap);
    std::printf("ok %s (%zu captured uploads)\n", name, snap.size());
}

void capture_tune()
{
    const char* name = "capture_tune";
    setenv("OCS_AUTOTUNE", "1", 1);
    cudaStream_t cap;
    check(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) == cudaSuccess, name, "stream");
    // a window and size class not tuned before: outside a capture this request would time variants
    std::vector<float> x = make_signal(700000, 77);
    const char* opts = "--nuttall_window --half_complex_return";
    ocs_geometry g;
    check(ocs_geometry_get(x.size(), 9, 0.25f, opts, &g) == OCS_OK, name, "geometry");
    float* d_in = nullptr;
    float* d_out = nullptr;
    check(cudaMalloc(&d_in, x.size() * 4) == cudaSuccess && cudaMalloc(&d_out, g.out_floats * 4) == cudaSuccess, name,
          "alloc");
    std::memcpy(d_in, x.data(), x.size() * 4);
    fake::capturing = cap;
    fake::event_fail_after = 0;  // a timing attempt would fail the call
    const int rc = ocs_activate_device(d_in, x.size(), 9, 0.25f, opts, d_out, g.out_floats, cap);
    fake::event_fail_after = -1;
    fake::capturing = nullptr;
    check(rc == OCS_OK, name, "rc " + std::to_string(rc));
    cudaStreamSynchronize(cap);
    check(std::memcmp(d_out, expected_out(x.data(), x.size(), 9, 0.25f, opts).data(), g.out_floats * 4) == 0, name,
          "result");
    cudaFree(d_in);
    cudaFree(d_out);
    cudaStreamDestroy(cap);
    setenv("OCS_AUTOTUNE", "0", 1);
    std::printf("ok %s\n", name);
}

void plan_tune()
{
    const char* name = "plan_tune";
    setenv("OCS_AUTOTUNE", "1", 1);
    int v = -7;
    // a key not tuned before: the call times the variants and reports the choice
    check(ocs_plan_tune(3000000, 10, 0.5f, "--blackman_window --remove_dc", &v) == OCS_OK, name, "tune");
    check(v >= 0 && v <= 4, name, "variant " + std::to_string(v));
    // again (the plan's tables are cached by now): the same choice, no scratch kept
    const long allocs0 = fake::live_allocs.load();
    int v2 = -7;
    check(ocs_plan_tune(3000000, 10, 0.5f, "--blackman_window --remove_dc", &v2) == OCS_OK && v2 == v, name,
          "second call");
    check(fake::live_allocs.load() == allocs0, name, "scratch left behind");
    // the tuned request then runs with that choice and the expected result
    std::vector<float> x = make_signal(3000000, 5);
    ocs_geometry g;
    check(ocs_geometry_get(x.size(), 10, 0.5f, "--blackman_window --remove_dc", &g) == OCS_OK, name, "geometry");
    std::vector<float> out(g.out_floats);
    uint64_t len = 0;
    check(ocs_activate(x.data(), x.size(), 10, 0.5f, "--blackman_window --remove_dc", out.data(), out.size(), &len) ==
              OCS_OK,
          name, "activate");
    check(std::memcmp(out.data(), expected_out(x.data(), x.size(), 10, 0.5f, "--blackman_window --remove_dc").data(),
                      out.size() * 4) == 0,
          name, "result");
    // one form only: windows above 2^15; and the option errors of ocs_activate
    check(ocs_plan_tune(1 << 20, 16, 0.5f, "--hamming_window", &v) == OCS_OK && v == -1, name, "large window");
    check(ocs_plan_tune(1 << 20, 10, 1.5f, "--hamming_window", &v) == OCS_EINVAL && v == -1, name, "bad overlap");
    setenv("OCS_AUTOTUNE", "0", 1);
    std::printf("ok %s\n", name);
}

void shutdown()
{
    const char* name = "shutdown";
    ocs_shutdown();
    check(fake::live_allocs.load() == 0, name, "device allocations left: " + std::to_string(fake::live_allocs.load()));
    check(fake::live_host_allocs.load() == 0, name, "pinned allocations left");
    check(fake::live_streams.load() == 0, name, "streams left: " + std::to_string(fake::live_streams.load()));
    check(fake::live_events.load() == 0, name, "events left: " + std::to_string(fake::live_events.load()));
    // and the runner starts again
    std::vector<float> x = make_signal(20000, 5), out;
    ocs_geometry g;
    check(ocs_geometry_get(x.size(), 9, 0.5f, "", &g) == OCS_OK, name, "geometry");
    out.resize(g.out_floats);
    uint64_t len = 0;
    check(ocs_activate(x.data(), x.size(), 9, 0.5f, "", out.data(), out.size(), &len) == OCS_OK, name, "again");
    check(std::memcmp(out.data(), expected_out(x.data(), x.size(), 9, 0.5f, "").data(), out.size() * 4) == 0, name,
          "result after re-initialisation");
    ocs_shutdown();
    std::printf("ok %s\n", name);
}

}  // namespace

// one request whose window and size class need a kernel-variant choice
int tune_cache_request()
{
    std::vector<float> x = make_signal(300000, 42);
    ocs_geometry g;
    if (ocs_geometry_get(x.size(), 10, 0.5f, "--hamming_window", &g) != OCS_OK) return OCS_EINVAL;
    std::vector<float> out(g.out_floats);
    uint64_t len = 0;
    const int rc = ocs_activate(x.data(), x.size(), 10, 0.5f, "--hamming_window", out.data(), out.size(), &len);
    if (rc == OCS_OK &&
        std::memcmp(out.data(), expected_out(x.data(), x.size(), 10, 0.5f, "--hamming_window").data(),
                    out.size() * 4) != 0)
        return -1;
    return rc;
}

int tune_cache(const std::string& mode, const char* file)
{
    setenv("OCS_AUTOTUNE", "1", 1);
    setenv("OCS_TUNE_CACHE", file, 1);
    check(ocs_init(0) == OCS_OK, "tune_cache", "ocs_init");
    if (mode == "tune-cache-read") {
        // the slot's own events first; after that no event can be created
        std::vector<float> x = make_signal(100, 1), out(1 << 12);
        uint64_t len = 0;
        check(ocs_activate(x.data(), x.size(), 6, 0.5f, "", out.data(), out.size(), &len) == OCS_OK, "tune_cache",
              "warm");
        fake::event_fail_after = 0;
    }
    const int rc = tune_cache_request();
    check(rc == OCS_OK, "tune_cache", mode + ": rc " + std::to_string(rc));
    ocs_shutdown();
    std::printf("ok %s\n", mode.c_str());
    return 0;
}

int main(int argc, char** argv)
{
    if (argc == 3) return tune_cache(argv[1], argv[2]);
    setenv("OCS_AUTOTUNE", "0", 1);
    setup_fail();
    table_fail();
    slot_fail();
    tune_fail();
    capture_tune();  // before any check that tunes other keys
    plan_tune();
    activate();
    concurrent();
    batch();
    batch_tune();
    capture();
    shutdown();
    std::printf("all ok\n");
    return 0;
}
