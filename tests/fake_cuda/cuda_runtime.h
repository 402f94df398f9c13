// TEST INFRASTRUCTURE ONLY: a host-only stand-in for the CUDA runtime calls
// the library's host code makes (occastft_gb300/csrc/ocs_server.cpp and
// ocs_api.cpp), so that code can be compiled unchanged and exercised on a
// machine without a GPU.  A stream is a FIFO worker thread; "device" memory is
// host memory; copies, host functions and stand-in kernels run in stream
// order; events order work across streams as CUDA events do.  Knobs for
// injecting failures and delays live in fake_control.h.
#pragma once
#include <cstddef>

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };
enum cudaStreamCaptureStatus {
    cudaStreamCaptureStatusNone = 0,
    cudaStreamCaptureStatusActive = 1,
    cudaStreamCaptureStatusInvalidated = 2
};
enum cudaFuncAttribute { cudaFuncAttributeMaxDynamicSharedMemorySize = 8 };
#define cudaStreamNonBlocking 0x01u
#define cudaEventDisableTiming 0x02u
#define cudaHostAllocPortable 0x01u
#define cudaHostAllocMapped 0x02u
#define cudaHostRegisterPortable 0x01u
#define CUDART_CB

struct alignas(8) float2 {
    float x, y;
};

struct cudaDeviceProp {
    char name[256];
    int major, minor;
    int multiProcessorCount;
};

struct FakeStream;
typedef FakeStream* cudaStream_t;
struct FakeEvent;
typedef FakeEvent* cudaEvent_t;
typedef void (*cudaHostFn_t)(void*);

cudaError_t cudaGetDevice(int* device);
cudaError_t cudaSetDevice(int device);
cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int device);
cudaError_t cudaDeviceSynchronize(void);
cudaError_t cudaMemGetInfo(size_t* free_bytes, size_t* total_bytes);
cudaError_t cudaMalloc(void** p, size_t bytes);
cudaError_t cudaFree(void* p);
cudaError_t cudaMallocAsync(void** p, size_t bytes, cudaStream_t st);
cudaError_t cudaFreeAsync(void* p, cudaStream_t st);
cudaError_t cudaHostAlloc(void** p, size_t bytes, unsigned flags);
cudaError_t cudaFreeHost(void* p);
cudaError_t cudaHostGetDevicePointer(void** d, void* h, unsigned flags);
cudaError_t cudaHostRegister(void* p, size_t bytes, unsigned flags);
cudaError_t cudaHostUnregister(void* p);
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* st, unsigned flags);
cudaError_t cudaStreamDestroy(cudaStream_t st);
cudaError_t cudaStreamSynchronize(cudaStream_t st);
cudaError_t cudaStreamIsCapturing(cudaStream_t st, cudaStreamCaptureStatus* status);
cudaError_t cudaStreamWaitEvent(cudaStream_t st, cudaEvent_t ev, unsigned flags);
cudaError_t cudaEventCreate(cudaEvent_t* ev);
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* ev, unsigned flags);
cudaError_t cudaEventDestroy(cudaEvent_t ev);
cudaError_t cudaEventRecord(cudaEvent_t ev, cudaStream_t st);
cudaError_t cudaEventSynchronize(cudaEvent_t ev);
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t start, cudaEvent_t end);
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st);
cudaError_t cudaMemsetAsync(void* dst, int value, size_t bytes, cudaStream_t st);
cudaError_t cudaLaunchHostFunc(cudaStream_t st, cudaHostFn_t fn, void* arg);
cudaError_t cudaGetLastError(void);
const char* cudaGetErrorString(cudaError_t e);

// typed forms, as the C++ runtime API offers them
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t bytes)
{
    return cudaMalloc(reinterpret_cast<void**>(p), bytes);
}
template <class T>
inline cudaError_t cudaHostAlloc(T** p, size_t bytes, unsigned flags)
{
    return cudaHostAlloc(reinterpret_cast<void**>(p), bytes, flags);
}
template <class T>
inline cudaError_t cudaHostGetDevicePointer(T** d, void* h, unsigned flags)
{
    return cudaHostGetDevicePointer(reinterpret_cast<void**>(d), h, flags);
}
template <class F>
inline cudaError_t cudaFuncSetAttribute(F, cudaFuncAttribute, int)
{
    return cudaSuccess;
}
