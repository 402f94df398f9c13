// TEST INFRASTRUCTURE ONLY: the request server (ocs_server.cpp) on the C
// ABI's real batch path (ocs_api.cpp: request parsing, tile lists, the
// descriptor staging each server slot reuses), against the host CUDA
// stand-in and stand-in kernels in this folder, with random delays on every
// stream.  Six threads submit 40 requests each (windows 2^6 .. 2^16, mixed
// overlaps and layouts) through a 4 MiB device pool and three slots; every
// result must equal the stand-in kernels' rule, the statistics must add up,
// and stopping the server and shutting the runner down must release every
// allocation, stream and event.  Prints "ok <name>" per check, "FAIL ..." and
// exit 1 on the first failure.
#include "../../include/occastft_gb300.h"
#include "fake_control.h"
#include "fake_expect.h"

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

struct Req {
    std::vector<float> x, out;
    int exp = 0;
    float ov = 0.0f;
    std::string opts;
    uint64_t ticket = 0;
    int status = -1;
};

}  // namespace

int main()
{
    const char* name = "served_batches";
    setenv("OCS_AUTOTUNE", "0", 1);
    fake::jitter_us = 100;
    ocs_server_config cfg{4u << 20, 32, 3};
    check(ocs_server_start(&cfg) == OCS_OK, name, "start");
    const char* opts[] = {"--hanning_window", "--hamming_window --half_complex_return",
                          "--blackman_window --layout=dense", "--hanning_window --half_complex_return --layout=dense",
                          "--remove_dc --serial_power"};
    const int exps[] = {6, 7, 8, 9, 10, 11, 12, 13, 14, 16};
    const float ovs[] = {0.0f, 0.25f, 0.5f, 0.75f, 0.3f};
    std::vector<std::vector<Req>> per(6);
    std::vector<std::thread> th;
    for (int t = 0; t < 6; ++t) {
        th.emplace_back([&, t] {
            std::mt19937 rng(31 + t);
            for (int i = 0; i < 40; ++i) {
                Req r;
                r.exp = exps[rng() % 10];
                r.ov = ovs[rng() % 5];
                r.opts = opts[rng() % 5];
                const uint64_t N = 1ull << r.exp;
                r.x = fake::make_signal(N / 2 + rng() % (r.exp == 16 ? 2 * N : 40000), 5000 + 100 * t + i);
                ocs_geometry g;
                check(ocs_geometry_get(r.x.size(), r.exp, r.ov, r.opts.c_str(), &g) == OCS_OK, name, "geometry");
                r.out.assign(g.out_floats, -7.0f);
                per[t].push_back(std::move(r));
            }
            for (auto& r : per[t])
                check(ocs_server_submit(r.x.data(), r.x.size(), r.exp, r.ov, r.opts.c_str(), r.out.data(),
                                        r.out.size(), &r.ticket) == OCS_OK,
                      name, "submit");
            for (auto& r : per[t]) check(ocs_server_wait(r.ticket, -1, &r.status) == OCS_OK, name, "wait");
        });
    }
    for (auto& t : th) t.join();
    fake::jitter_us = 0;
    int n = 0;
    for (auto& v : per)
        for (auto& r : v) {
            const std::string tag = "exp " + std::to_string(r.exp) + " ov " + std::to_string(r.ov) + " n " +
                                    std::to_string(r.x.size()) + " '" + r.opts + "'";
            check(r.status == OCS_OK, name, tag + ": status " + std::to_string(r.status));
            const std::vector<float> want = fake::expected_out(r.x.data(), r.x.size(), r.exp, r.ov, r.opts);
            check(std::memcmp(r.out.data(), want.data(), r.out.size() * 4) == 0, name, tag + ": result differs");
            ++n;
        }
    ocs_server_stats st;
    check(ocs_server_get_stats(&st) == OCS_OK, name, "stats");
    check(st.completed == 240 && st.failed == 0 && st.pool_used == 0, name, "statistics");
    check(st.batches < st.completed, name, "no requests were coalesced");
    std::printf("ok %s (%d requests in %llu batches)\n", name, n, (unsigned long long)st.batches);

    const char* name2 = "release";
    check(ocs_server_stop() == OCS_OK, name2, "stop");
    ocs_shutdown();
    check(fake::live_allocs.load() == 0, name2, "device allocations left: " + std::to_string(fake::live_allocs.load()));
    check(fake::live_host_allocs.load() == 0, name2, "pinned allocations left");
    check(fake::live_streams.load() == 0, name2, "streams left: " + std::to_string(fake::live_streams.load()));
    check(fake::live_events.load() == 0, name2, "events left: " + std::to_string(fake::live_events.load()));
    std::printf("ok %s\n", name2);
    std::printf("all ok\n");
    return 0;
}
