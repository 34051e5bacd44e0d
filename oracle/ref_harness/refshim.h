// Forced-include shim used only when compiling the unmodified reference
// sources (Calc.cu) with CUDA 13.  CUDA 13 removed five cudaDeviceProp
// fields that the reference's queryGpus() prints (Calc.cu:28-38).  The shim
// substitutes a struct that carries those fields and fills them from
// cudaDeviceGetAttribute, so the reference compiles without a source edit.
#pragma once
#include <cuda_runtime.h>

struct cbref_device_prop : public cudaDeviceProp {
    int clockRate;
    int memoryClockRate;
    int deviceOverlap;
    int kernelExecTimeoutEnabled;
};

static inline cudaError_t cbref_get_device_properties(cbref_device_prop* p, int dev) {
    cudaError_t e = cudaGetDeviceProperties(static_cast<cudaDeviceProp*>(p), dev);
    p->clockRate = p->memoryClockRate = p->deviceOverlap = p->kernelExecTimeoutEnabled = 0;
    cudaDeviceGetAttribute(&p->clockRate, cudaDevAttrClockRate, dev);
    cudaDeviceGetAttribute(&p->memoryClockRate, cudaDevAttrMemoryClockRate, dev);
    cudaDeviceGetAttribute(&p->deviceOverlap, cudaDevAttrGpuOverlap, dev);
    cudaDeviceGetAttribute(&p->kernelExecTimeoutEnabled, cudaDevAttrKernelExecTimeout, dev);
    return e;
}

#define cudaDeviceProp cbref_device_prop
#define cudaGetDeviceProperties cbref_get_device_properties
