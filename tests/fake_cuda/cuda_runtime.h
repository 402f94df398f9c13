// TEST INFRASTRUCTURE ONLY: a host-only stand-in for the few CUDA runtime
// calls the request server (occastft_gb300/csrc/ocs_server.cpp) makes, so its
// control logic (admission, coalescing, completion, cancellation, statistics,
// start/stop from several threads) can be compiled unchanged and exercised on
// a machine without a GPU.  A stream is a FIFO worker thread; "device" memory
// is host memory; copies and host functions run in stream order.  Knobs for
// injecting failures live in fake_control.h.
#pragma once
#include <cstddef>

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2 };
#define cudaStreamNonBlocking 0x01u
#define CUDART_CB

struct FakeStream;
typedef FakeStream* cudaStream_t;
struct FakeEvent;
typedef FakeEvent* cudaEvent_t;
typedef void (*cudaHostFn_t)(void*);

cudaError_t cudaGetDevice(int* device);
cudaError_t cudaSetDevice(int device);
cudaError_t cudaMemGetInfo(size_t* free_bytes, size_t* total_bytes);
cudaError_t cudaMalloc(void** p, size_t bytes);
cudaError_t cudaFree(void* p);
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* st, unsigned flags);
cudaError_t cudaStreamDestroy(cudaStream_t st);
cudaError_t cudaStreamSynchronize(cudaStream_t st);
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st);
cudaError_t cudaLaunchHostFunc(cudaStream_t st, cudaHostFn_t fn, void* arg);
cudaError_t cudaGetLastError(void);
const char* cudaGetErrorString(cudaError_t e);
