// TEST INFRASTRUCTURE ONLY: drives the request server's C ABI
// (ocs_server_*, occastft_gb300/csrc/ocs_server.cpp compiled unchanged)
// against the host-only CUDA stand-in in this folder.  Each check prints
// "ok <name>"; the first failure prints "FAIL <name>: <why>" and exits 1.
//
//   admission   4 threads x 100 requests through a pool that holds a few at a
//               time: every output correct, requests coalesced, pool drained
//   copy_error  a request whose input copy cannot be issued ends OCS_ECUDA,
//               the rest of its group completes
//   cancel      a queued request is withdrawn; one already admitted is not
//   stop_race   a stop while 6 threads submit and wait: no use after free
//               (run under ThreadSanitizer), every accepted request written
//   start_fail  a start that fails part-way releases its pool and streams
#include "../../include/occastft_gb300.h"
#include "fake_control.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <mutex>
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

struct Req {
    std::vector<float> in, out;
    int exp = 6;
    float ov = 0.5f;
    std::string opts;
    uint64_t ticket = 0;
    int status = -1;
};

Req make_req(std::mt19937& rng, uint64_t n_max)
{
    Req r;
    const uint64_t n = 64 + rng() % (n_max - 63);
    r.in.resize(n);
    for (auto& v : r.in) v = (float)(rng() % 2001) / 1000.0f - 1.0f;
    r.exp = 6 + (int)(rng() % 3);
    r.ov = (rng() % 2) ? 0.5f : 0.25f;
    r.opts = (rng() % 2) ? "--hanning_window" : "--hamming_window --half_complex_return";
    ocs_geometry g;
    check(ocs_geometry_get(n, r.exp, r.ov, r.opts.c_str(), &g) == OCS_OK, "make_req", "geometry");
    r.out.assign(g.out_floats, -12345.0f);
    return r;
}

bool correct(const Req& r)
{
    for (uint64_t k = 0; k < r.out.size(); ++k)
        if (r.out[k] != fake::expected(r.in.data(), r.in.size(), r.exp, k)) return false;
    return true;
}

int submit(Req& r)
{
    return ocs_server_submit(r.in.data(), r.in.size(), r.exp, r.ov, r.opts.c_str(), r.out.data(), r.out.size(),
                             &r.ticket);
}

void leak_check(const char* name)
{
    check(fake::live_allocs.load() == 0, name, "device allocations left: " + std::to_string(fake::live_allocs.load()));
    check(fake::live_streams.load() == 0, name, "streams left: " + std::to_string(fake::live_streams.load()));
}

void admission()
{
    const char* name = "admission";
    fake::kernel_us = 300;
    ocs_server_config cfg{256u << 10, 16, 3};  // 256 KiB pool: a handful of requests at a time
    check(ocs_server_start(&cfg) == OCS_OK, name, "start");
    check(ocs_server_start(&cfg) == OCS_EINVAL, name, "a second start must be refused");
    const long launches0 = fake::launches.load();
    std::vector<std::vector<Req>> per(4);
    std::vector<std::thread> th;
    for (int t = 0; t < 4; ++t) {
        th.emplace_back([&, t] {
            std::mt19937 rng(100 + t);
            for (int i = 0; i < 100; ++i) per[t].push_back(make_req(rng, 4096));
            for (auto& r : per[t]) check(submit(r) == OCS_OK, name, "submit");
            for (auto& r : per[t]) check(ocs_server_wait(r.ticket, -1, &r.status) == OCS_OK, name, "wait");
        });
    }
    for (auto& t : th) t.join();
    for (auto& v : per)
        for (auto& r : v) {
            check(r.status == OCS_OK, name, "status " + std::to_string(r.status));
            check(correct(r), name, "output differs from the stand-in kernel's");
        }
    ocs_server_stats st;
    check(ocs_server_get_stats(&st) == OCS_OK, name, "stats");
    check(st.completed == 400 && st.failed == 0, name, "completed " + std::to_string(st.completed));
    check(st.batches < 400 && fake::launches.load() - launches0 == (long)st.batches, name,
          "batches " + std::to_string(st.batches));
    check(fake::max_launch_requests.load() > 1, name, "no launch coalesced requests");
    check(st.pool_used == 0 && st.pending == 0, name, "pool not drained");
    check(st.p50_ms > 0 && st.p99_ms >= st.p50_ms && st.max_ms >= st.p99_ms, name, "latency order");
    check(ocs_server_reset_stats() == OCS_OK, name, "reset");
    check(ocs_server_get_stats(&st) == OCS_OK && st.completed == 0 && st.max_ms == 0, name, "reset stats");
    check(ocs_server_stop() == OCS_OK, name, "stop");
    leak_check(name);
    std::printf("ok %s (%llu batches for 400 requests)\n", name, (unsigned long long)fake::launches.load());
}

void copy_error()
{
    const char* name = "copy_error";
    fake::kernel_us = 2000;  // the group forms while the first launch runs
    ocs_server_config cfg{256u << 10, 16, 3};
    check(ocs_server_start(&cfg) == OCS_OK, name, "start");
    std::mt19937 rng(7);
    std::vector<Req> rs;
    for (int i = 0; i < 10; ++i) rs.push_back(make_req(rng, 2048));
    fake::fail_copy_ptr = rs[6].in.data();
    for (auto& r : rs) check(submit(r) == OCS_OK, name, "submit");
    for (auto& r : rs) check(ocs_server_wait(r.ticket, -1, &r.status) == OCS_OK, name, "wait");
    fake::fail_copy_ptr = nullptr;
    for (int i = 0; i < 10; ++i) {
        if (i == 6) {
            check(rs[i].status == OCS_ECUDA, name, "failed copy reported " + std::to_string(rs[i].status));
            check(rs[i].out[0] == -12345.0f, name, "a failed request's output was written");
        } else {
            check(rs[i].status == OCS_OK && correct(rs[i]), name, "request " + std::to_string(i));
        }
    }
    ocs_server_stats st;
    check(ocs_server_get_stats(&st) == OCS_OK && st.failed == 1 && st.completed == 9, name, "stats");
    check(ocs_server_stop() == OCS_OK, name, "stop");
    leak_check(name);
    std::printf("ok %s\n", name);
}

void cancel()
{
    const char* name = "cancel";
    fake::kernel_us = 50000;  // the last of six requests stays queued for 250 ms
    ocs_server_config cfg{1u << 20, 1, 1};  // one request per launch, one in flight
    check(ocs_server_start(&cfg) == OCS_OK, name, "start");
    std::mt19937 rng(9);
    std::vector<Req> rs;
    for (int i = 0; i < 6; ++i) rs.push_back(make_req(rng, 1024));
    for (auto& r : rs) check(submit(r) == OCS_OK, name, "submit");
    check(ocs_server_cancel(rs[5].ticket) == OCS_OK, name, "cancel a queued request");
    check(ocs_server_wait(rs[5].ticket, 0, nullptr) == OCS_EINVAL, name, "a withdrawn ticket must be unknown");
    check(ocs_server_wait(rs[0].ticket, -1, &rs[0].status) == OCS_OK, name, "wait");
    check(ocs_server_cancel(rs[0].ticket) == OCS_EINVAL, name, "a finished request cannot be withdrawn");
    for (int i = 1; i < 5; ++i) check(ocs_server_wait(rs[i].ticket, -1, &rs[i].status) == OCS_OK, name, "wait");
    for (int i = 0; i < 5; ++i) check(rs[i].status == OCS_OK && correct(rs[i]), name, "request");
    check(rs[5].out[0] == -12345.0f, name, "a withdrawn request ran");
    check(ocs_server_stop() == OCS_OK, name, "stop");
    leak_check(name);
    std::printf("ok %s\n", name);
}

void stop_race()
{
    const char* name = "stop_race";
    fake::kernel_us = 200;
    ocs_server_config cfg{1u << 20, 32, 3};
    check(ocs_server_start(&cfg) == OCS_OK, name, "start");
    std::mutex mu;
    std::vector<Req*> accepted;
    std::atomic<int> refused{0}, waits_after_stop{0};
    std::vector<std::thread> th;
    std::vector<std::vector<Req>> store(6);
    for (int t = 0; t < 6; ++t) {
        store[t].reserve(100000);
        th.emplace_back([&, t] {
            std::mt19937 rng(500 + t);
            for (;;) {
                store[t].push_back(make_req(rng, 1024));
                Req& r = store[t].back();
                const int rc = submit(r);
                if (rc != OCS_OK) {
                    check(rc == OCS_EINVAL, name, "submit during stop: code " + std::to_string(rc));
                    ++refused;
                    return;
                }
                {
                    std::lock_guard<std::mutex> lk(mu);
                    accepted.push_back(&r);
                }
                const int w = ocs_server_wait(r.ticket, -1, &r.status);
                if (w == OCS_OK) {
                    check(r.status == OCS_OK, name, "status");
                } else {
                    check(w == OCS_EINVAL, name, "wait during stop: code " + std::to_string(w));
                    ++waits_after_stop;
                    r.status = OCS_OK;  // finished by the stop's drain; checked below
                }
            }
        });
    }
    std::this_thread::sleep_for(std::chrono::milliseconds(50));
    check(ocs_server_stop() == OCS_OK, name, "stop");
    for (auto& t : th) t.join();
    check(refused.load() == 6, name, "every client must see the server gone");
    for (Req* r : accepted) check(correct(*r), name, "an accepted request was not finished by the stop");
    check(ocs_server_submit(nullptr, 0, 6, 0.5f, "", nullptr, 0, nullptr) == OCS_EINVAL, name, "after stop");
    leak_check(name);
    std::printf("ok %s (%zu requests accepted, %d waits ended by the stop)\n", name, accepted.size(),
                waits_after_stop.load());
}

void start_fail()
{
    const char* name = "start_fail";
    fake::stream_fail_after = 2;  // the third slot's stream cannot be created
    ocs_server_config cfg{1u << 20, 8, 3};
    check(ocs_server_start(&cfg) == OCS_ECUDA, name, "start must fail");
    fake::stream_fail_after = -1;
    leak_check(name);
    check(ocs_server_stop() == OCS_EINVAL, name, "nothing to stop");
    check(ocs_server_start(&cfg) == OCS_OK, name, "start after a failed start");
    check(ocs_server_stop() == OCS_OK, name, "stop");
    leak_check(name);
    std::printf("ok %s\n", name);
}

}  // namespace

// no arguments: every check; otherwise the named ones
int main(int argc, char** argv)
{
    const struct {
        const char* name;
        void (*fn)();
    } checks[] = {{"admission", admission}, {"copy_error", copy_error}, {"cancel", cancel},
                  {"stop_race", stop_race}, {"start_fail", start_fail}};
    for (const auto& c : checks) {
        bool want = argc < 2;
        for (int i = 1; i < argc; ++i) want |= std::string(argv[i]) == c.name;
        if (want) c.fn();
    }
    std::printf("all ok\n");
    return 0;
}
