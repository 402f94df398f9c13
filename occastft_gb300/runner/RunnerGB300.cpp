// Vendor half of the GB300 runner: Genv, Gcodes, InitEnv, BuildKernel, UnInit
// and ActivateSTFT — the pieces the reference's CUDA runner defines in
// StandAlone/cross_gpgpu/CUDA/src/CudaImpl.cpp:285-510.
//
// ActivateSTFT runs the whole pipeline as the fused GB300 kernel through
// ocs_activate (host vectors in and out, copies overlapped with compute)
// instead of the reference's allocate / copy / seven launches / copy / free.
// Like the CUDA runner it returns std::nullopt when the pipeline status is not
// "OK" (CudaImpl.cpp:497-501); the status is kept in last_status.
#include "gb300Struct.hpp"
#include "occastft_gb300.h"
#include "occastft_runner.hpp"

#include <cstdlib>

void Runner::InitEnv()
{
    env = new Genv;
    kens = new Gcodes;
    const char* d = std::getenv("OCS_DEVICE");
    env->device = d ? std::atoi(d) : 0;
}

void Runner::BuildKernel()
{
    if (ocs_init(env->device) != OCS_OK) last_status = ocs_last_error();
}

void Runner::UnInit() { ocs_shutdown(); }

MAYBE_DATA
Runner::ActivateSTFT(VECF& inData, const int& windowSizeEXP, const float& overlapRatio, const std::string& options)
{
    ocs_geometry g;
    int rc = ocs_geometry_get(inData.size(), windowSizeEXP, overlapRatio, options.c_str(), &g);
    if (rc != OCS_OK) {
        last_status = ocs_last_error();
        return std::nullopt;
    }
    VECF out(g.out_floats);
    uint64_t len = 0;
    rc = ocs_activate(inData.data(), inData.size(), windowSizeEXP, overlapRatio, options.c_str(), out.data(),
                      out.size(), &len);
    if (rc != OCS_OK) {
        last_status = ocs_last_error();
        return std::nullopt;
    }
    last_status = "OK";
    return out;
}
