// TEST INFRASTRUCTURE ONLY: the library internals the request server
// (occastft_gb300/csrc/ocs_server.cpp) links against, for compiling it
// without a GPU and without the C ABI (ocs_api.cpp): a stand-in batch launch,
// error text and geometry.  Geometry and option parsing are the library's
// own (ocs_host.cpp, linked beside this file); only the device work is
// replaced.
#include "cuda_runtime.h"
#include "fake_control.h"
#include "ocs_host.h"
#include "ocs_internal.h"

#include <chrono>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {
thread_local std::string t_err;
}  // namespace

namespace ocs {
void set_last_error(const std::string& msg) { t_err = msg; }

namespace internal {

// The batch launch: validates each request as the library does and queues one
// unit of stream work that writes fake::expected() into every output.
int batch_enqueue(ocs_request* reqs, int count, cudaStream_t st, BatchScratch&, bool)
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
    fake::enqueue(st, [items, us] {
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
