// userStruct of the GB300 runner's runnerFunction hooks: the stream every
// hook launches on (the reference's CUDA runner passes a cudaData with its
// stream, StandAlone/cross_gpgpu/CUDA/include/cudaStruct.hpp).
#pragma once

struct GB300Data {
    void* stream = nullptr;  // cudaStream_t; nullptr = legacy default stream
};

// The runner's environment and kernel set (Runner::env, Runner::kens).  The
// fused kernels are compiled ahead of time for sm_103a; plans (twiddle and
// window tables, launch shapes) are built on first use and cached by the
// C ABI, so the kernel set holds nothing.
struct Genv {
    int device = 0;
};

struct Gcodes {
};
