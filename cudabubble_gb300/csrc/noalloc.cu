// Allocation-free volume integral of a device-resident real field.
//
// cb_intf_noalloc computes (mean(u) + addition) * multiply * volume, the
// quantity of the reference's Calc::intf (Calc.cu:191-262; its callers in
// phasefield.cpp:286, :313, :322 take the volume with addition 1, multiply
// 1/2, the surface area of the s-term with addition 0, multiply 3/(2 sqrt 2),
// the elastic energy of f^2 with addition 0, multiply 1/(2 eps)).  The
// reference, and the per-plane reduction of the stepper's xy pass, keep the
// partial sums in memory owned by the caller or the instance; this variant
// keeps them in one file-scope __device__ array instead, so it never
// allocates.  Callers that may not allocate device
// memory -- code running inside a memory pool that is already carved up, a
// host that forbids driver allocations after start-up, a step issued between
// other work on a budgeted device -- can still reduce a field.
//
// Shape of the computation: one CTA per z-plane sums its ny*nx values in a
// fixed order into scratch.part[z]; the last CTA to finish (an atomic
// counter in the same scratch) sums the nz partials, writes the result and
// puts the counter back to zero, so the result does not depend on which CTA
// finished last and two calls in a row give the same bits.
#include <cuda_runtime.h>

#include "cb_fft.cuh"
#include "stepper.cuh"

namespace cb {
namespace {

constexpr int kNoAllocMaxPlanes = 4096;  // partial sums held by the scratch (32 KiB)
constexpr int kNoAllocMaxDevices = 64;
constexpr int kNoAllocThreads = 256;

struct NoAllocScratch {
    double part[kNoAllocMaxPlanes];
    unsigned count;  // CTAs done in the current call; must be 0 between calls
    unsigned pad[63];
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

__global__ void __launch_bounds__(kNoAllocThreads)
intf_noalloc_kernel(const double* __restrict__ u, int nz, long long plane, double addition, double scale,
                    NoAllocScratch* scr, double* __restrict__ val) {
    __shared__ double red[2 * 32 + 2];
    const int z = blockIdx.x;
    const double* src = u + (size_t)z * (size_t)plane;
    double s = 0.0;
    for (long long i = threadIdx.x; i < plane; i += kNoAllocThreads) s += __ldg(src + i);
    double v[1] = {s}, sum[1];
    block_sum<1>(v, sum, red);
    int* last = reinterpret_cast<int*>(red + 64);
    if (threadIdx.x == 0) {
        scr->part[z] = sum[0];
        __threadfence();
        const unsigned done = atomicAdd(&scr->count, 1u);
        *last = done == (unsigned)(nz - 1);
    }
    __syncthreads();
    if (!*last) return;
    __threadfence();
    double tot[1];
    block_sum_parts<1>(scr->part, nz, tot, red);
    if (threadIdx.x == 0) {
        const double n = (double)nz * (double)plane;
        *val = (tot[0] / n + addition) * scale;
        scr->count = 0u;  // ready for the next call
    }
}

std::mutex g_noalloc_mu;
NoAllocScratch* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// The scratch address of the current device, resolved on every call (it does not
// allocate): a cached address goes stale when the device's context is rebuilt
// (cudaDeviceReset, a new primary context).  The first call that sees an address
// for a device -- once per device and context -- clears the counter
// synchronously, so that first call must not be made while a stream is being
// captured.
int noalloc_scratch(NoAllocScratch** out) {
    int dev = 0;
    CB_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return fail(CB_EINVAL, "cb_intf_noalloc: device %d beyond the %d supported", dev, kNoAllocMaxDevices);
    void* p = nullptr;
    CB_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    NoAllocScratch* s = static_cast<NoAllocScratch*>(p);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (g_noalloc_ptr[dev] != s) {
        CB_CK(cudaMemset(&s->count, 0, sizeof(unsigned)));
        CB_CK(cudaDeviceSynchronize());
        g_noalloc_ptr[dev] = s;
    }
    *out = s;
    return CB_OK;
}

}  // namespace
}  // namespace cb

extern "C" int cb_intf_noalloc(const double* d_u, int nx, int ny, int nz, double addition, double multiply,
                               double volume, double* d_val, void* stream) {
    using namespace cb;
    if (!d_u || !d_val) return fail(CB_EINVAL, "cb_intf_noalloc: null device pointer");
    if (nx < 1 || ny < 1 || nz < 1) return fail(CB_EINVAL, "cb_intf_noalloc: bad grid %dx%dx%d", nx, ny, nz);
    if (nz > kNoAllocMaxPlanes)
        return fail(CB_EINVAL, "cb_intf_noalloc: nz = %d exceeds the scratch maximum of %d planes", nz,
                    kNoAllocMaxPlanes);
    NoAllocScratch* scr = nullptr;
    if (int rc = noalloc_scratch(&scr)) return rc;
    const long long plane = (long long)nx * (long long)ny;
    intf_noalloc_kernel<<<nz, kNoAllocThreads, 0, static_cast<cudaStream_t>(stream)>>>(d_u, nz, plane, addition,
                                                                                      multiply * volume, scr, d_val);
    CB_CK(cudaGetLastError());
    return CB_OK;
}
