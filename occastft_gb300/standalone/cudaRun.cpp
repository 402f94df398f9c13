// cudaRun: the GB300 runner executable that the reference's proxy launches.
//
// Drop-in for the reference's per-backend runner binary (main and
// Runner::ServerInit in StandAlone/cross_gpgpu/GLOBAL/RunnerCommon.cpp:62-164;
// launched as `<dir>/cudaRun <port>` by RuntimeCheck::ExcuteRunner,
// StandAlone/src/runtimeChecker.cpp:19-31).  It serves WebSocket clients on
// 0.0.0.0:<port> (default 54500):
//   * binary message: one RequestCapnp.  The signal is read from the POSIX
//     shared memory object it names (result written back over it) or from
//     its data list (result returned in the data list).  The answer copies the
//     request's fields except options and data; a failure answers with
//     sharedMemory = "ERR" (FFTStruct.cpp:16-22);
//   * text "CLOSE_REQUEST": answers "CLOSE_COMPLETE" and stops the runner.
// Each request runs the fused GB300 pipeline through the C ABI.  Differences
// from the reference, on purpose: a data-list request that follows a
// shared-memory request gets its result in the data list (the reference keeps
// the previous request's unmapped pointer and writes through it); results
// that do not fit the shared memory region, or a data list longer than a
// Cap'n Proto list can hold (2^29 - 1 elements), answer "ERR" instead of
// writing past the region.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "occastft_gb300.h"
#include "request_codec.hpp"
#include "shm_payload.hpp"
#include "ws_server.hpp"

using namespace ocs_standalone;

namespace {

bool g_log = false;

// How a shared-memory payload is prepared for the device copies:
// pin: page-locked for the request (cudaHostRegister), the default;
// populate: page tables built at map time, copies through the driver's
// pageable path; plain: neither.  OCS_CUDARUN_SHM=pin|populate|plain.
enum class ShmMode { pin, populate, plain };
ShmMode g_shm_mode = ShmMode::pin;

// Runs the pipeline on host memory through ocs_activate (copies in chunks,
// overlapped with the kernels).  in and out may be the same region (the
// shared-memory case): ocs_activate then writes each part of the result only
// after the input it overwrites has reached the device.
std::string run_pipeline(const float* in, uint64_t n, int exp, float ov, const std::string& opts, float* out,
                         uint64_t out_cap_floats)
{
    ocs_geometry g;
    if (ocs_geometry_get(n, exp, ov, opts.c_str(), &g) != OCS_OK) return ocs_last_error();
    if (g.out_floats > out_cap_floats) return "result larger than the shared memory region";
    uint64_t len = 0;
    if (ocs_activate(in, n, exp, ov, opts.c_str(), out, out_cap_floats, &len) != OCS_OK) return ocs_last_error();
    return "";
}

// the answer's fields: the request's, except options and data (MakeWField,
// FFTStruct.cpp:95-110)
Request answer_of(const Request& q)
{
    Request a;
    a.windowRadix = q.windowRadix;
    a.overlapRatio = q.overlapRatio;
    a.mappedID = q.mappedID;
    a.sharedMemory = q.sharedMemory;
    a.memPTR = q.memPTR;
    a.posixFileDes = q.posixFileDes;
    a.windowsHandlePTR = q.windowsHandlePTR;
    a.dataLength = q.dataLength;
    a.overlapdataLength = q.overlapdataLength;
    return a;
}

void send_answer(Connection& c, const Request& a)
{
    std::vector<uint64_t> buf((encoded_size(a) + 7) / 8);
    encode_request(a, reinterpret_cast<uint8_t*>(buf.data()), nullptr);
    c.send_binary(reinterpret_cast<const uint8_t*>(buf.data()), encoded_size(a));
}

constexpr uint64_t kMaxListElements = (1ull << 29) - 1;

void handle_request(Connection& c, const Message& m)
{
    const auto t0 = std::chrono::steady_clock::now();
    Request q;
    std::vector<float> scratch;
    const std::string derr = decode_request(m.data(), m.size, q, scratch);
    if (!derr.empty()) {
        Request a;
        a.sharedMemory = "ERR";
        send_answer(c, a);
        if (g_log) std::fprintf(stderr, "cudaRun: undecodable request: %s\n", derr.c_str());
        return;
    }
    Request a = answer_of(q);
    const int exp = (int)q.windowRadix;
    std::string status;
    const char* path = "none";
    if (!q.sharedMemory.empty()) {
        path = "shm";
        if (q.sharedMemory == "ERR") {
            status = "request marked ERR";
        } else if (!protocol_shm_name(q.sharedMemory)) {
            status = "shared memory name is not of the form /STFT<mappedID>SHAREDMEM";
        } else {
            ShmMapping map;
            status = shm_map(q.sharedMemory, q.overlapdataLength, map, g_shm_mode == ShmMode::populate);
            if (status.empty() && q.dataLength > map.bytes / sizeof(float))
                status = "dataLength floats exceed the shared memory region";
            bool pinned = false;
            if (status.empty() && g_shm_mode == ShmMode::pin)
                pinned = ocs_host_register(map.ptr, map.bytes) == OCS_OK;  // unpinned still works, slower
            if (status.empty()) {
                float* p = static_cast<float*>(map.ptr);
                status = run_pipeline(p, q.dataLength, exp, q.overlapRatio, q.options, p, map.bytes / sizeof(float));
            }
            if (pinned) ocs_host_unregister(map.ptr);
            shm_unmap(map);
        }
        if (!status.empty()) a.sharedMemory = "ERR";
        send_answer(c, a);
    } else if (q.dataCount) {
        path = "list";
        ocs_geometry g;
        if (ocs_geometry_get(q.dataCount, exp, q.overlapRatio, q.options.c_str(), &g) != OCS_OK) {
            status = ocs_last_error();
        } else if (g.out_floats > kMaxListElements) {
            status = "result longer than a Cap'n Proto list can hold";
        } else {
            // the result goes straight into the answer's data list
            a.dataCount = g.out_floats;
            a.dataLength = g.out_floats;
            a.data = nullptr;
            std::vector<uint64_t> buf((encoded_size(a) + 7) / 8);
            float* slot = nullptr;
            encode_request(a, reinterpret_cast<uint8_t*>(buf.data()), &slot);
            status = run_pipeline(q.data, q.dataCount, exp, q.overlapRatio, q.options, slot, g.out_floats);
            if (status.empty()) c.send_binary(reinterpret_cast<const uint8_t*>(buf.data()), encoded_size(a));
        }
        if (!status.empty()) {
            a = answer_of(q);
            a.sharedMemory = "ERR";
            send_answer(c, a);
        }
    } else {
        status = "request without data";
        a.sharedMemory = "ERR";
        send_answer(c, a);
    }
    if (g_log) {
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        std::fprintf(stderr, "cudaRun: id=%s path=%s n=%llu exp=%d ov=%g opts='%s' %s (%.3f ms)\n", q.mappedID.c_str(),
                     path, (unsigned long long)(q.sharedMemory.empty() ? q.dataCount : q.dataLength), exp,
                     (double)q.overlapRatio, q.options.c_str(), status.empty() ? "OK" : status.c_str(), ms);
    }
}

}  // namespace

int main(int argc, char* argv[])
{
    int port = 54500;  // the reference's default port
    if (argc == 2) {
        char* end = nullptr;
        const long v = std::strtol(argv[1], &end, 10);
        if (end == argv[1] || *end != '\0' || v < 0 || v > 65535) {
            std::fprintf(stderr, "cudaRun: bad port '%s'\n", argv[1]);
            return 1;
        }
        port = (int)v;
    }
    const char* lg = std::getenv("OCS_CUDARUN_LOG");
    g_log = lg && lg[0] == '1';
    if (const char* sm = std::getenv("OCS_CUDARUN_SHM")) {
        if (!std::strcmp(sm, "populate")) g_shm_mode = ShmMode::populate;
        else if (!std::strcmp(sm, "plain")) g_shm_mode = ShmMode::plain;
    }
    // listen first: a proxy may connect while the device initialises (its
    // connection waits in the backlog until the serve loop accepts it)
    WsServer server;
    const std::string err = server.listen(port);
    if (!err.empty()) {
        std::fprintf(stderr, "ERR on server init: %s\n", err.c_str());
        return 1;
    }
    const char* dev = std::getenv("OCS_DEVICE");
    if (ocs_init(dev ? std::atoi(dev) : 0) != OCS_OK)
        std::fprintf(stderr, "cudaRun: device init failed (%s); requests will answer ERR\n", ocs_last_error());
    if (g_log) std::fprintf(stderr, "cudaRun: listening on 0.0.0.0:%d\n", server.port());
    server.run([&](Connection& c, const Message& m) {
        if (m.binary) {
            handle_request(c, m);
        } else if (m.text() == "CLOSE_REQUEST") {
            c.send_text("CLOSE_COMPLETE");
            server.stop();
        }
    });
    ocs_shutdown();
    return 0;
}
