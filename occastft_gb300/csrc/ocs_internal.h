// Library-internal interface shared by the C ABI (ocs_api.cpp) and the
// request server (ocs_server.cpp).  Not exported.
#pragma once
#include "../../include/occastft_gb300.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <string>

namespace ocs {
namespace internal {

// Descriptor scratch of one in-flight batch: pinned staging + device copy.
struct BatchScratch {
    char* host = nullptr;
    size_t host_cap = 0;
    char* dev = nullptr;
    size_t dev_cap = 0;
    cudaEvent_t staged = nullptr;  // descriptors have left the staging buffer
    cudaEvent_t done = nullptr;    // the kernel that read the device copy has finished
};

int batch_scratch_grow(BatchScratch& b, size_t bytes);
void batch_scratch_release(BatchScratch& b);
int batch_prepare_into(const ocs_request* reqs, int count, BatchScratch& b);
// tune: time the tile lengths on this call when the batch's mix is new
// (ocs_batch_device outside capture; the server never tunes)
int batch_enqueue(ocs_request* reqs, int count, cudaStream_t st, BatchScratch& b, bool tune = false);
int ensure_ready();
// drops the no-allocation batch's per-device set-up (ocs_shutdown)
void noalloc_forget_devices();
void set_error(int code, const std::string& msg);

}  // namespace internal
}  // namespace ocs
