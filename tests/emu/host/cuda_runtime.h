// Test infrastructure: the CUDA runtime calls of the stepper's host code (stepper.cuh,
// launch_impl.cuh) over host memory, for tests/test_host_emulation.py.  Streams run
// their work at once, a capture records closures that a graph launch replays, kernels
// run through emu::launch (one OS thread per CUDA thread), and a launch asking for more
// than 48 KB of dynamic shared memory fails unless the kernel's limit was raised.
#pragma once
#include "../fake/cuda_runtime.h"

// ---------------------------------------------------------------- runtime API
#include <functional>
enum cudaErrorEnum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaErrorMemoryAllocation = 2,
                     cudaErrorLaunchFailure = 719, cudaErrorIllegalAddress = 700 };
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2,
                      cudaMemcpyDeviceToDevice = 3, cudaMemcpyDefault = 4 };
enum cudaFuncAttribute { cudaFuncAttributeMaxDynamicSharedMemorySize = 8 };
enum cudaStreamCaptureMode { cudaStreamCaptureModeGlobal = 0, cudaStreamCaptureModeThreadLocal = 1,
                             cudaStreamCaptureModeRelaxed = 2 };
#define cudaStreamNonBlocking 1
#define cudaEventDisableTiming 2
namespace emu {
struct Stream;
struct Event;
struct Graph;
}
typedef emu::Stream* cudaStream_t_;
#define cudaStream_t cudaStream_t_
typedef emu::Event* cudaEvent_t;
typedef emu::Graph* cudaGraph_t;
typedef emu::Graph* cudaGraphExec_t;
namespace emu {
cudaError_t launch_kernel(dim3 g, dim3 b, size_t smem, cudaStream_t s, const void* fn, int clus,
                          std::function<void()> body);
cudaError_t set_attr(const void* fn, int attr, int v);
}
cudaError_t cudaGetLastError();
const char* cudaGetErrorString(cudaError_t e);
cudaError_t cudaMalloc(void** p, size_t n);
template <class T> inline cudaError_t cudaMalloc(T** p, size_t n) { return cudaMalloc((void**)p, n); }
cudaError_t cudaFree(void* p);
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind k);
cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind k, cudaStream_t st = 0);
cudaError_t cudaMemsetAsync(void* d, int v, size_t n, cudaStream_t st = 0);
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, unsigned f);
cudaError_t cudaStreamDestroy(cudaStream_t s);
cudaError_t cudaStreamSynchronize(cudaStream_t s);
cudaError_t cudaDeviceSynchronize();
cudaError_t cudaEventCreate(cudaEvent_t* e);
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, unsigned f);
cudaError_t cudaStreamWaitEvent(cudaStream_t s, cudaEvent_t e, unsigned f = 0);
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s = 0);
cudaError_t cudaEventSynchronize(cudaEvent_t e);
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b);
cudaError_t cudaEventDestroy(cudaEvent_t e);
cudaError_t cudaGetDevice(int* d);
cudaError_t cudaStreamBeginCapture(cudaStream_t s, cudaStreamCaptureMode m);
cudaError_t cudaStreamEndCapture(cudaStream_t s, cudaGraph_t* g);
cudaError_t cudaGraphInstantiate(cudaGraphExec_t* e, cudaGraph_t g, unsigned long long flags);
cudaError_t cudaGraphLaunch(cudaGraphExec_t e, cudaStream_t s);
cudaError_t cudaGraphExecDestroy(cudaGraphExec_t e);
cudaError_t cudaGraphDestroy(cudaGraph_t g);
template <class F> inline cudaError_t cudaFuncSetAttribute(F* fn, cudaFuncAttribute a, int v) {
    return emu::set_attr((const void*)fn, (int)a, v);
}
