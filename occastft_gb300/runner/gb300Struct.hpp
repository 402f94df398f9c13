// userStruct of the GB300 runner's runnerFunction hooks: the stream every
// hook launches on (the reference's CUDA runner passes a cudaData with its
// stream, StandAlone/cross_gpgpu/CUDA/include/cudaStruct.hpp).
#pragma once

struct GB300Data {
    void* stream = nullptr;  // cudaStream_t; nullptr = legacy default stream
};
