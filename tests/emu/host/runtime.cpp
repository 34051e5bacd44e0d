// Test infrastructure (tests/test_host_emulation.py): the emulated CUDA runtime of
// cuda_runtime.h beside this file.  Host memory, streams that run their work at once,
// graphs as recorded closures, kernels run by emu::launch with one OS thread per CUDA
// thread of a cluster, reused for every cluster of the grid.
#include <sys/mman.h>
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <thread>
#include <vector>

#include "cuda_runtime.h"

namespace emu {
thread_local Block* t_blk = nullptr;
thread_local dim3 t_tid, t_bid;
dim3 g_bdim, g_gdim;
std::mutex g_atomic_mu;
static thread_local cudaError_t t_last = cudaSuccess;
static std::map<const void*, int> g_attr;
static long g_launches = 0;

struct Stream {
    bool capturing = false;
    std::vector<std::function<void()>>* cap = nullptr;
};
struct Event {
    double t = 0;
};
struct Graph {
    std::vector<std::function<void()>> nodes;
};

static double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// EMU_GUARD set: device buffers and shared memory are placed at the end of their own
// mapping, between two 64 MB inaccessible regions, so an access far outside every
// allocation (beyond AddressSanitizer's redzones, into another live allocation) faults
static const size_t kGuard = (size_t)64 << 20;
static bool guarded() {
    static const bool g = getenv("EMU_GUARD") != nullptr;
    return g;
}
static std::map<void*, std::pair<void*, size_t>> g_maps;
static std::mutex g_map_mu;
void* emu_alloc(size_t n, size_t align) {
    if (!guarded()) return malloc(n ? n : 1);
    const size_t pg = (size_t)sysconf(_SC_PAGESIZE);
    const size_t na = ((n ? n : 1) + align - 1) / align * align;
    const size_t body = (na + pg - 1) / pg * pg;
    const size_t total = kGuard + body + kGuard;
    char* base = (char*)mmap(nullptr, total, PROT_NONE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (base == MAP_FAILED) abort();
    if (mprotect(base + kGuard, body, PROT_READ | PROT_WRITE)) abort();
    void* p = base + kGuard + body - na;
    std::lock_guard<std::mutex> lk(g_map_mu);
    g_maps[p] = {base, total};
    return p;
}
void emu_free(void* p) {
    if (!guarded()) {
        free(p);
        return;
    }
    std::lock_guard<std::mutex> lk(g_map_mu);
    auto it = g_maps.find(p);
    if (it == g_maps.end()) return;
    munmap(it->second.first, it->second.second);
    g_maps.erase(it);
}

void launch(dim3 grid, int nt, size_t smem, int clus, const std::function<void()>& body) {
    g_bdim = dim3(nt);
    g_gdim = grid;
    const int total = nt * clus;
    Cluster cl;
    std::vector<Block> blocks(clus);
    for (int r = 0; r < clus; ++r) {
        blocks[r].ex = new double[nt];
        blocks[r].smem = (unsigned char*)emu_alloc(smem, 16);
        blocks[r].smem_bytes = smem;
        blocks[r].rank = r;
        blocks[r].cl = &cl;
        cl.blocks[r] = &blocks[r];
    }
    auto reset = [&] {
        cl.bar.alive = total;
        cl.bar.arrived = 0;
        for (int r = 0; r < clus; ++r) {
            blocks[r].bar.alive = nt;
            blocks[r].bar.arrived = 0;
            for (auto& nb : blocks[r].named) nb.alive = nb.arrived = 0;
            for (int w = 0; w < 32; ++w) {
                blocks[r].warp[w].alive = std::max(0, std::min(32, nt - 32 * w));
                blocks[r].warp[w].arrived = 0;
            }
            memset(blocks[r].smem, 0xA5, smem);
        }
    };
    reset();
    Barrier pool;
    pool.alive = total;
    std::vector<std::thread> th;
    th.reserve(total);
    for (int t = 0; t < total; ++t)
        th.emplace_back([&, t] {
            const int r = t / nt;
            for (unsigned by = 0; by < grid.y; ++by)
                for (unsigned bx = 0; bx < grid.x; bx += clus) {
                    t_blk = &blocks[r];
                    t_tid = dim3(t % nt);
                    t_bid = dim3(bx + r, by);
                    body();
                    blocks[r].bar.drop();
                    blocks[r].warp[(t % nt) >> 5].drop();
                    cl.bar.drop();
                    pool.wait();  // every thread is done with this cluster
                    if (t == 0) reset();
                    pool.wait();
                }
        });
    for (auto& x : th) x.join();
    for (auto& b : blocks) {
        emu_free(b.smem);
        delete[] b.ex;
    }
}

cudaError_t launch_kernel(dim3 g, dim3 b, size_t smem, cudaStream_t s, const void* fn, int clus,
                          std::function<void()> body) {
    if (b.x > 1024 || b.x == 0 || g.x == 0 || g.y == 0) {
        fprintf(stderr, "EMU: bad launch grid %u,%u block %u\n", g.x, g.y, b.x);
        return t_last = cudaErrorInvalidValue;
    }
    if (smem > 48 * 1024) {
        auto it = g_attr.find(fn);
        if (it == g_attr.end() || (size_t)it->second < smem) {
            fprintf(stderr, "EMU: launch with %zu B dynamic smem above the function's limit (%d)\n", smem,
                    it == g_attr.end() ? 49152 : it->second);
            return t_last = cudaErrorInvalidValue;
        }
    }
    if (smem > 227 * 1024) {
        fprintf(stderr, "EMU: smem %zu above 227 KB\n", smem);
        return t_last = cudaErrorInvalidValue;
    }
    const int nt = (int)b.x;
    auto run = [=]() {
        ++g_launches;
        if (getenv("EMU_TRACE"))
            fprintf(stderr, "EMU: launch %ld grid %u,%u block %d smem %zu clus %d\n", g_launches, g.x, g.y, nt, smem,
                    clus);
        launch(g, nt, smem, clus, body);
    };
    if (s && s->capturing) s->cap->push_back(run);
    else run();
    return t_last = cudaSuccess;
}
cudaError_t set_attr(const void* fn, int attr, int v) {
    if (attr == cudaFuncAttributeMaxDynamicSharedMemorySize) {
        if (v > 227 * 1024) return cudaErrorInvalidValue;
        g_attr[fn] = v;
    }
    return cudaSuccess;
}
}  // namespace emu

using emu::Stream;

cudaError_t cudaGetLastError() {
    cudaError_t e = emu::t_last;
    emu::t_last = cudaSuccess;
    return e;
}
const char* cudaGetErrorString(cudaError_t e) { return e ? "emulated error" : "no error"; }
cudaError_t cudaMalloc(void** p, size_t n) {
    *p = emu::emu_alloc(n, 256);
    memset(*p, 0xEE, n);
    return cudaSuccess;
}
cudaError_t cudaFree(void* p) {
    emu::emu_free(p);
    return cudaSuccess;
}
static void check_capture(cudaStream_t s, const char* what) {
    if (s && s->capturing) {
        fprintf(stderr, "EMU: %s inside capture\n", what);
        abort();
    }
}
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
    memcpy(d, s, n);
    return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind, cudaStream_t st) {
    check_capture(st, "memcpy");
    memcpy(d, s, n);
    return cudaSuccess;
}
cudaError_t cudaMemsetAsync(void* d, int v, size_t n, cudaStream_t st) {
    check_capture(st, "memset");
    memset(d, v, n);
    return cudaSuccess;
}
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, unsigned) {
    *s = new Stream;
    return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t s) {
    delete s;
    return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t s) {
    check_capture(s, "stream sync");
    return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
cudaError_t cudaEventCreate(cudaEvent_t* e) {
    *e = new emu::Event;
    return cudaSuccess;
}
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, unsigned) { return cudaEventCreate(e); }
// streams run their work at once, so every wait is already satisfied
cudaError_t cudaStreamWaitEvent(cudaStream_t s, cudaEvent_t, unsigned) {
    check_capture(s, "event wait");
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s) {
    check_capture(s, "event record");
    e->t = emu::now_ms();
    return cudaSuccess;
}
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b) {
    *ms = (float)(b->t - a->t);
    return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t e) {
    delete e;
    return cudaSuccess;
}
cudaError_t cudaGetDevice(int* d) {
    *d = 0;
    return cudaSuccess;
}
cudaError_t cudaStreamBeginCapture(cudaStream_t s, cudaStreamCaptureMode) {
    if (!s || s->capturing) return cudaErrorInvalidValue;
    s->capturing = true;
    s->cap = new std::vector<std::function<void()>>;
    return cudaSuccess;
}
cudaError_t cudaStreamEndCapture(cudaStream_t s, cudaGraph_t* g) {
    if (!s || !s->capturing) return cudaErrorInvalidValue;
    *g = new emu::Graph{*s->cap};
    delete s->cap;
    s->cap = nullptr;
    s->capturing = false;
    return cudaSuccess;
}
cudaError_t cudaGraphInstantiate(cudaGraphExec_t* e, cudaGraph_t g, unsigned long long) {
    *e = new emu::Graph{g->nodes};
    return cudaSuccess;
}
cudaError_t cudaGraphLaunch(cudaGraphExec_t e, cudaStream_t s) {
    check_capture(s, "graph launch");
    if (getenv("EMU_TRACE")) fprintf(stderr, "EMU: graph launch (%zu nodes)\n", e->nodes.size());
    for (auto& f : e->nodes) f();
    return cudaSuccess;
}
cudaError_t cudaGraphExecDestroy(cudaGraphExec_t e) {
    delete e;
    return cudaSuccess;
}
cudaError_t cudaGraphDestroy(cudaGraph_t g) {
    delete g;
    return cudaSuccess;
}
