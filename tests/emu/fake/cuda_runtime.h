// Test infrastructure: a host emulation of the CUDA subset the stepper's kernel
// headers use, so that tests/test_kernel_emulation.py can run the kernels' index
// arithmetic on the CPU under AddressSanitizer.  Every CUDA thread is an OS thread;
// __syncthreads, warp shuffles and cluster barriers are real barriers.  Not part of
// the library: the product path runs only the sm_103a build.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <mutex>
#include <thread>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __cluster_dims__(...)
#define __align__(n) alignas(n)
// a kernel's static shared variable: one object for the whole launch, which is one block's
// as the emulation runs the blocks of a one-CTA-cluster launch one at a time (no kernel
// with a cluster of two declares one)
#define __shared__ static

struct float2 { float x, y; };
struct alignas(16) float4 { float x, y, z, w; };
struct alignas(16) double2 { double x, y; };
struct dim3 {
    unsigned x = 1, y = 1, z = 1;
    dim3() {}
    dim3(unsigned a, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
inline float2 make_float2(float a, float b) { return {a, b}; }
inline float4 make_float4(float a, float b, float c, float d) { float4 r; r.x = a; r.y = b; r.z = c; r.w = d; return r; }
inline double2 make_double2(double a, double b) { double2 r; r.x = a; r.y = b; return r; }
using std::isfinite;
using std::min;
using std::max;

namespace emu {
struct Barrier {
    std::mutex mu;
    std::condition_variable cv;
    int alive = 0, arrived = 0;
    long gen = 0;
    void wait() {
        std::unique_lock<std::mutex> lk(mu);
        const long g = gen;
        if (++arrived == alive) {
            arrived = 0;
            ++gen;
            cv.notify_all();
        } else {
            cv.wait(lk, [&] { return gen != g; });
        }
    }
    void drop() {
        std::unique_lock<std::mutex> lk(mu);
        --alive;
        if (arrived > 0 && arrived == alive) {
            arrived = 0;
            ++gen;
            cv.notify_all();
        }
    }
};
struct Block {
    Barrier bar;
    Barrier named[16];  // bar.sync id, n: the group barriers of the persistent batched kernel
    Barrier warp[32];   // the warps' shuffles
    double* ex = nullptr;  // shuffle exchange, one slot per thread
    unsigned char* smem = nullptr;
    size_t smem_bytes = 0;
    int rank = 0;
    struct Cluster* cl = nullptr;
};
struct Cluster {
    Barrier bar;
    Block* blocks[2] = {nullptr, nullptr};
};
extern thread_local Block* t_blk;
extern thread_local dim3 t_tid, t_bid;
extern dim3 g_bdim, g_gdim;
extern std::mutex g_atomic_mu;
}  // namespace emu

#define threadIdx (::emu::t_tid)
#define blockIdx (::emu::t_bid)
#define blockDim (::emu::g_bdim)
#define gridDim (::emu::g_gdim)

inline void __syncthreads() { emu::t_blk->bar.wait(); }
#define CB_EMULATION 1
namespace emu {
// named barrier `id` of this block over n threads: each generation takes the count of
// its first arrival, as bar.sync does (the same id serves groups of different sizes)
inline void named_sync(int id, int n) {
    Barrier& b = t_blk->named[id];
    std::unique_lock<std::mutex> lk(b.mu);
    if (b.arrived == 0) b.alive = n;
    const long g = b.gen;
    if (++b.arrived == b.alive) {
        b.arrived = 0;
        ++b.gen;
        b.cv.notify_all();
    } else {
        b.cv.wait(lk, [&] { return b.gen != g; });
    }
}
}  // namespace emu
inline void __threadfence() { std::atomic_thread_fence(std::memory_order_seq_cst); }
template <class T> inline T __ldg(const T* p) { return *p; }
template <class T> inline T __ldcg(const T* p) { return *p; }
inline unsigned atomicAdd(unsigned* p, unsigned v) {
    std::lock_guard<std::mutex> lk(emu::g_atomic_mu);
    const unsigned o = *p;
    *p = o + v;
    return o;
}
template <class T> inline T __shfl_xor_sync(unsigned, T v, int o) {
    emu::Block* b = emu::t_blk;
    const int t = (int)threadIdx.x;
    emu::Barrier& w = b->warp[t >> 5];  // a warp-wide exchange, as on the device
    b->ex[t] = (double)v;
    w.wait();
    const T r = (T)b->ex[t ^ o];
    w.wait();
    return r;
}
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __double2float_rn(double d) { return (float)d; }
inline float2 __fadd2_rn(float2 a, float2 b) { return {a.x + b.x, a.y + b.y}; }
inline float2 __fmul2_rn(float2 a, float2 b) { return {a.x * b.x, a.y * b.y}; }
inline float2 __ffma2_rn(float2 a, float2 b, float2 c) { return {fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y)}; }

typedef int cudaError_t;
typedef struct emu_stream_* cudaStream_t;  // declarations only (the kernel drivers launch through emu::launch)
inline void __nanosleep(unsigned) { std::this_thread::yield(); }
