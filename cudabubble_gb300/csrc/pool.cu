// Batched and served pools of stepper instances.
//
// Instances that share (grid, method, coefficient mode) form a size class.
// A class owns a fixed-capacity device table of instance descriptors; one
// launch per pass covers every slot of the class (blockIdx.y = slot), and one
// captured CUDA graph runs one attempt of every class, each class on its own
// forked stream.  An empty slot points at a control block that is always
// done, so its CTAs return at once; admitting or retiring an instance only
// rewrites one table entry and the graph is never re-captured.  Every slot
// keeps its own dt, accept/reject state and FP64 scalars, so an instance's
// result is the same alone and in any mix.
//
// The reference runs one grid per process (main.cpp:17-18) and has no batched
// or served mode; these are additions of this implementation.
#include <chrono>
#include <deque>
#include <iterator>
#include <map>
#include <thread>
#include <type_traits>

#include "mega.h"
#include "stepper.cuh"

namespace cb {

struct SlotSummary {
    int done, status, steps, attempts, rejects, pad;
    double E, dt;
};

template <class T>
__global__ void gather_kernel(const InstT<T>* __restrict__ table, int cap, SlotSummary* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    const Ctrl* c = table[i].ctrl;
    SlotSummary s;
    s.done = c->done;
    s.status = c->status;
    s.steps = c->steps;
    s.attempts = c->attempts;
    s.rejects = c->rejects;
    s.pad = 0;
    s.E = c->E_state;
    s.dt = c->dt;
    out[i] = s;
}

// phi0 = tanh(d / (sqrt(2) eps)) of one ellipsoid or the union of two
// (d = max(d1, d2)), on the grid x_i = i L / n - L / 2 (fluidbase.cpp:156-161).
__global__ void ellipsoid_kernel(double* __restrict__ out, int nx, int nz, double L, double eps, double a0,
                                 double a1, double a2, double c0, double c1, double c2, double b0, double b1,
                                 double b2, double e0, double e1, double e2) {
    const size_t n = (size_t)nx * nx * nz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % nx), y = (int)((i / nx) % nx), z = (int)(i / ((size_t)nx * nx));
        const double X = x * L / nx - L / 2.0, Y = y * L / nx - L / 2.0, Z = z * L / nz - L / 2.0;
        const double u = (X - c0) / a0, v = (Y - c1) / a1, w = (Z - c2) / a2;
        double d = (1.0 - sqrt(u * u + v * v + w * w)) * fmin(a0, fmin(a1, a2));
        if (b0 > 0) {
            const double u2 = (X - e0) / b0, v2 = (Y - e1) / b1, w2 = (Z - e2) / b2;
            d = fmax(d, (1.0 - sqrt(u2 * u2 + v2 * v2 + w2 * w2)) * fmin(b0, fmin(b1, b2)));
        }
        out[i] = tanh(d / (sqrt(2.0) * eps));
    }
}

template <class T> struct PoolClass {
    int nx = 0, nz = 0, method = 0, accurate = 0, cap = 0, ntiles = 0, split = 0, curv = 0;
    InstT<T>* table = nullptr;
    SlotSummary* sum = nullptr;
    std::vector<Stepper<T>*> occ;
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

template <class T> class Pool {
   public:
    ~Pool() {
        if (st) cudaStreamSynchronize(st);
        if (g) cudaGraphExecDestroy(g);
        for (auto& c : cls) {
            cudaFree(c.table);
            cudaFree(c.sum);
            if (c.s) cudaStreamDestroy(c.s);
            if (c.fork) cudaEventDestroy(c.fork);
            if (c.join) cudaEventDestroy(c.join);
        }
        cudaFree(dummy_ctrl);
        cudaFreeHost(h_sum);
        cudaFree(m_tasks);
        cudaFree(m_insts);
        cudaFree(m_need);
        cudaFree(m_done);
        cudaFree(m_err);
        if (st) cudaStreamDestroy(st);
    }

    int init() {
        CB_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        CB_CK(cudaMalloc(&dummy_ctrl, sizeof(Ctrl)));
        Ctrl c;
        memset(&c, 0, sizeof c);
        c.done = 1;
        CB_CK(cudaMemcpy(dummy_ctrl, &c, sizeof c, cudaMemcpyHostToDevice));
        memset(&dummy, 0, sizeof dummy);
        dummy.ctrl = dummy_ctrl;
        return CB_OK;
    }

    int find(int nx, int nz, int method, int accurate, int split, int curv) const {
        for (size_t i = 0; i < cls.size(); ++i)
            if (cls[i].nx == nx && cls[i].nz == nz && cls[i].method == method && cls[i].accurate == accurate &&
                cls[i].split == split && cls[i].curv == curv)
                return (int)i;
        return -1;
    }

    int add_class(int nx, int nz, int method, int accurate, int split, int curv, int ntiles, int cap) {
        if (g) return fail(CB_EINVAL, "pool graph already built");
        PoolClass<T> c;
        c.nx = nx; c.nz = nz; c.method = method; c.accurate = accurate; c.cap = cap; c.ntiles = ntiles;
        c.split = split;
        c.curv = curv;
        c.occ.assign(cap, nullptr);
        CB_CK(cudaMalloc(&c.table, sizeof(InstT<T>) * cap));
        CB_CK(cudaMalloc(&c.sum, sizeof(SlotSummary) * cap));
        std::vector<InstT<T>> init(cap, dummy);
        CB_CK(cudaMemcpy(c.table, init.data(), sizeof(InstT<T>) * cap, cudaMemcpyHostToDevice));
        CB_CK(cudaStreamCreateWithFlags(&c.s, cudaStreamNonBlocking));
        CB_CK(cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming));
        CB_CK(cudaEventCreateWithFlags(&c.join, cudaEventDisableTiming));
        cls.push_back(c);
        return CB_OK;
    }

    // put an instance into a free slot of its class
    int place(Stepper<T>* sp, int* ci, int* si) {
        const Params& p = sp->params();
        const int c = find(p.nx, p.nz, p.method, sp->accurate(), p.split, p.curv);
        if (c < 0) return fail(CB_EINVAL, "no size class for %dx%dx%d", p.nx, p.ny, p.nz);
        for (int k = 0; k < cls[c].cap; ++k) {
            if (!cls[c].occ[k]) {
                cls[c].occ[k] = sp;
                CB_CK(cudaMemcpyAsync(cls[c].table + k, &sp->inst(), sizeof(InstT<T>), cudaMemcpyHostToDevice, st));
                CB_CK(cudaStreamSynchronize(st));
                *ci = c;
                *si = k;
                return CB_OK;
            }
        }
        return fail(CB_ENOMEM, "size class full");
    }

    bool has_free(int c) const {
        for (auto* o : cls[c].occ)
            if (!o) return true;
        return false;
    }

    int release(int c, int k) {
        cls[c].occ[k] = nullptr;
        CB_CK(cudaMemcpyAsync(cls[c].table + k, &dummy, sizeof(InstT<T>), cudaMemcpyHostToDevice, st));
        CB_CK(cudaStreamSynchronize(st));
        return CB_OK;
    }

    int build_graph() {
        int total = 0;
        for (auto& c : cls) total += c.cap;
        CB_CK(cudaMallocHost(&h_sum, sizeof(SlotSummary) * (total > 0 ? total : 1)));
        if (persistent) return build_mega_graph();
        cudaGraph_t gr = nullptr;
        CB_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        cudaError_t r = cudaSuccess;
        for (auto& c : cls) {
            if (r == cudaSuccess) r = cudaEventRecord(c.fork, st);
            if (r == cudaSuccess) r = cudaStreamWaitEvent(c.s, c.fork, 0);
            if (r == cudaSuccess)
                r = enqueue_group<T>(c.method, c.nx, c.nz, c.table, c.cap, c.ntiles, c.accurate, false, c.split,
                                     c.curv, c.s);
            if (r == cudaSuccess) r = cudaEventRecord(c.join, c.s);
            if (r == cudaSuccess) r = cudaStreamWaitEvent(st, c.join, 0);
        }
        cudaError_t e = cudaStreamEndCapture(st, &gr);
        if (r != cudaSuccess) {
            if (gr) cudaGraphDestroy(gr);
            return fail(CB_ECUDA, "pool capture: %s", cudaGetErrorString(r));
        }
        CB_CK(e);
        cudaError_t ie = cudaGraphInstantiate(&g, gr, 0);
        cudaGraphDestroy(gr);
        CB_CK(ie);
        return CB_OK;
    }

    // ---- the persistent batched attempt (mega.h): one kernel per attempt of every
    // instance instead of a launch per pass and class
    bool persistent = false;
    int mega_clusters = 0, mega_tasks = 0;

    int mega_check() const {
        if constexpr (!std::is_same<T, float>::value) {
            return fail(CB_EUNSUPPORTED, "persistent batch: FP32 form only");
        } else {
            for (auto& c : cls) {
                if (c.method != M_ETD2) return fail(CB_EUNSUPPORTED, "persistent batch: ETD-RK2 only");
                if (c.curv) return fail(CB_EUNSUPPORTED, "persistent batch: no spontaneous curvature");
                if (!mega_size_ok(c.nx) || !mega_size_ok(c.nz))
                    return fail(CB_EUNSUPPORTED, "persistent batch: grid %dx%dx%d not built into its kernel", c.nx,
                                c.nx, c.nz);
                const bool clus = mega_cluster_xy(c.nx);
                if (c.split == XYP_SPLIT || (clus && c.split == XYP_SINGLE) || (!clus && c.split == XYP_CLUSTER))
                    return fail(CB_EUNSUPPORTED,
                                "persistent batch: xy path %d of %d^2 planes not built into its kernel", c.split,
                                c.nx);
            }
            return CB_OK;
        }
    }

    // the work list (phase-major, larger grids first), the per-phase completion counts,
    // and a graph of one attempt: zero the counters, launch the persistent kernel
    int build_mega_graph() {
        int rc = mega_check();
        if (rc) return rc;
        std::vector<const InstT<float>*> ptrs;
        std::vector<MegaClass> mc;
        for (size_t c = 0; c < cls.size(); ++c) {
            mc.push_back(MegaClass{cls[c].nx, cls[c].nz, cls[c].accurate, cls[c].cap, (int)ptrs.size()});
            for (int k = 0; k < cls[c].cap; ++k) ptrs.push_back(reinterpret_cast<const InstT<float>*>(cls[c].table + k));
        }
        std::vector<MegaTask> tasks;
        std::vector<unsigned> need;
        mega_plan(mc, tasks, need);
        mega_tasks = (int)tasks.size();
        const int maxc = mega_max_clusters();
        if (maxc <= 0) return fail(CB_ECUDA, "persistent batch: no resident cluster of its kernel");
        mega_clusters = std::min(maxc, std::max(1, mega_tasks));
        CB_CK(cudaMalloc(&m_tasks, sizeof(MegaTask) * tasks.size()));
        CB_CK(cudaMalloc(&m_insts, sizeof(void*) * ptrs.size()));
        CB_CK(cudaMalloc(&m_need, sizeof(unsigned) * need.size()));
        CB_CK(cudaMalloc(&m_done, sizeof(unsigned) * (need.size() + 1)));  // + the unit counter
        CB_CK(cudaMalloc(&m_err, sizeof(unsigned)));
        CB_CK(cudaMemcpy(m_tasks, tasks.data(), sizeof(MegaTask) * tasks.size(), cudaMemcpyHostToDevice));
        CB_CK(cudaMemcpy(m_insts, ptrs.data(), sizeof(void*) * ptrs.size(), cudaMemcpyHostToDevice));
        CB_CK(cudaMemcpy(m_need, need.data(), sizeof(unsigned) * need.size(), cudaMemcpyHostToDevice));
        CB_CK(cudaMemset(m_err, 0, sizeof(unsigned)));
        MegaArgs a;
        memset(&a, 0, sizeof a);
        a.tasks = m_tasks;
        a.insts = m_insts;
        a.need = m_need;
        a.done = m_done;
        a.ticket = m_done + need.size();
        a.err = m_err;
        a.ntasks = mega_tasks;
        a.ninst = (int)ptrs.size();
        cudaGraph_t gr = nullptr;
        CB_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        cudaError_t r = cudaMemsetAsync(m_done, 0, sizeof(unsigned) * (need.size() + 1), st);
        if (r == cudaSuccess) r = mega_launch(a, mega_clusters, st);
        cudaError_t e = cudaStreamEndCapture(st, &gr);
        if (r != cudaSuccess) {
            if (gr) cudaGraphDestroy(gr);
            return fail(CB_ECUDA, "persistent batch capture: %s", cudaGetErrorString(r));
        }
        CB_CK(e);
        cudaError_t ie = cudaGraphInstantiate(&g, gr, 0);
        cudaGraphDestroy(gr);
        CB_CK(ie);
        return CB_OK;
    }

    // waits of the persistent kernel that ran out since the last call (synchronises)
    int mega_failures(unsigned* n) {
        *n = 0;
        if (!persistent) return CB_OK;
        CB_CK(cudaMemcpyAsync(n, m_err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        CB_CK(cudaStreamSynchronize(st));
        if (*n) CB_CK(cudaMemset(m_err, 0, sizeof(unsigned)));
        return CB_OK;
    }

    cudaError_t launch(int attempts) {
        for (int i = 0; i < attempts; ++i) {
            cudaError_t r = cudaGraphLaunch(g, st);
            if (r != cudaSuccess) return r;
        }
        return cudaSuccess;
    }

    // per-slot summaries of every class (class-major), synchronises the pool stream
    int poll(std::vector<SlotSummary>& out) {
        int off = 0;
        for (auto& c : cls) {
            gather_kernel<T><<<(c.cap + 127) / 128, 128, 0, st>>>(c.table, c.cap, c.sum);
            CB_CK(cudaGetLastError());
            CB_CK(cudaMemcpyAsync(h_sum + off, c.sum, sizeof(SlotSummary) * c.cap, cudaMemcpyDeviceToHost, st));
            off += c.cap;
        }
        CB_CK(cudaStreamSynchronize(st));
        out.assign(h_sum, h_sum + off);
        return CB_OK;
    }

    int slot_index(int c, int k) const {
        int off = 0;
        for (int i = 0; i < c; ++i) off += cls[i].cap;
        return off + k;
    }
    cudaStream_t stream() const { return st; }
    std::vector<PoolClass<T>> cls;

   private:
    cudaStream_t st = nullptr;
    cudaGraphExec_t g = nullptr;
    Ctrl* dummy_ctrl = nullptr;
    InstT<T> dummy{};
    SlotSummary* h_sum = nullptr;
    MegaTask* m_tasks = nullptr;
    const InstT<float>** m_insts = nullptr;
    unsigned* m_need = nullptr;
    unsigned* m_done = nullptr;
    unsigned* m_err = nullptr;
};

// ---------------------------------------------------------------- batch
struct BatchBase {
    virtual ~BatchBase() {}
    virtual int set_phi(int i, const double* phi, bool dev) = 0;
    virtual int get_phi(int i, double* phi, bool dev) = 0;
    virtual int scalars(int i, cb_scalars* s) = 0;
    virtual int run(int nsteps, cb_run_stats* st, long long flush_bytes, double* ms) = 0;
    virtual int size() const = 0;
};

template <class T> class Batch final : public BatchBase {
   public:
    ~Batch() override {
        pool.reset();
        items.clear();
        cudaFree(flush_buf);
    }
    int init(const cb_params* ps, int n, bool persistent = false) {
        pool.reset(new Pool<T>());
        int rc = pool->init();
        if (rc) return rc;
        pool->persistent = persistent;
        for (int i = 0; i < n; ++i) {
            std::unique_ptr<Stepper<T>> s(new Stepper<T>());
            rc = s->init(ps[i]);
            if (rc) return rc;
            items.push_back(std::move(s));
        }
        for (auto& it : items) {
            const Params& p = it->params();
            if (pool->find(p.nx, p.nz, p.method, it->accurate(), p.split, p.curv) >= 0) continue;
            int cap = 0;
            for (auto& jt : items) {
                const Params& q = jt->params();
                if (q.nx == p.nx && q.nz == p.nz && q.method == p.method && jt->accurate() == it->accurate() &&
                    q.split == p.split && q.curv == p.curv)
                    ++cap;
            }
            rc = pool->add_class(p.nx, p.nz, p.method, it->accurate(), p.split, p.curv, it->tiles(), cap);
            if (rc) return rc;
        }
        where.resize(n);
        for (int i = 0; i < n; ++i) {
            rc = pool->place(items[i].get(), &where[i].first, &where[i].second);
            if (rc) return rc;
        }
        return pool->build_graph();
    }
    int size() const override { return (int)items.size(); }
    int set_phi(int i, const double* phi, bool dev) override { return items[i]->set_phi(phi, dev); }
    int get_phi(int i, double* phi, bool dev) override { return items[i]->get_phi(phi, dev); }
    int scalars(int i, cb_scalars* s) override { return items[i]->scalars(s); }

    // every instance advances nsteps accepted steps (or stops on its own exit
    // test); flush_bytes > 0 times attempt by attempt with an L2 flush between
    int run(int nsteps, cb_run_stats* stt, long long flush_bytes, double* ms_out) override {
        int steps0 = 0, att0 = 0;
        for (auto& it : items) {
            cb_scalars s;
            int rc = it->scalars(&s);
            if (rc) return rc;
            steps0 += s.steps;
            att0 += s.attempts;
            rc = it->prepare_run(nsteps);
            if (rc) return rc;
        }
        if (flush_bytes > 0 && flush_bytes != flush_size) {
            cudaFree(flush_buf);
            flush_buf = nullptr;
            CB_CK(cudaMalloc(&flush_buf, (size_t)flush_bytes));
            flush_size = flush_bytes;
        }
        cudaStream_t s = pool->stream();
        cudaEvent_t e0, e1;
        CB_CK(cudaEventCreate(&e0));
        CB_CK(cudaEventCreate(&e1));
        double total = 0.0;
        int launches = 0;
        const long long limit = 70LL * (nsteps + 1) * 2 + 1000;
        std::vector<SlotSummary> sum;
        bool all = false;
        CB_CK(cudaEventRecord(e0, s));
        while (!all && launches < limit) {
            const int chunk = flush_bytes > 0 ? 1 : 8;
            if (flush_bytes > 0) {
                CB_CK(cudaMemsetAsync(flush_buf, launches & 0xff, (size_t)flush_bytes, s));
                CB_CK(cudaEventRecord(e0, s));
            }
            CB_CK(pool->launch(chunk));
            launches += chunk;
            if (flush_bytes > 0) {
                CB_CK(cudaEventRecord(e1, s));
                CB_CK(cudaEventSynchronize(e1));
                float m = 0.f;
                cudaEventElapsedTime(&m, e0, e1);
                total += m;
            }
            int rc = pool->poll(sum);
            if (rc) return rc;
            unsigned lost = 0;
            rc = pool->mega_failures(&lost);
            if (rc) return rc;
            if (lost) return fail(CB_ETIMEOUT, "persistent batch: %u dependency waits ran out", lost);
            all = true;
            for (auto& w : where)
                if (!sum[pool->slot_index(w.first, w.second)].done) { all = false; break; }
        }
        if (flush_bytes <= 0) {
            CB_CK(cudaEventRecord(e1, s));
            CB_CK(cudaEventSynchronize(e1));
            float m = 0.f;
            cudaEventElapsedTime(&m, e0, e1);
            total = m;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        int steps1 = 0, att1 = 0, worst = ST_TARGET;
        for (auto& it : items) {
            int status = 0;
            int rc = it->finish_run(&status);
            if (rc) return rc;
            cb_scalars sc;
            it->scalars(&sc);
            steps1 += sc.steps;
            att1 += sc.attempts;
            if (status != ST_TARGET) worst = status;
        }
        if (stt) {
            stt->steps = steps1 - steps0;
            stt->attempts = att1 - att0;
            stt->status = worst;
            stt->graph_launches = launches;
            stt->device_ms = total;
        }
        if (ms_out) *ms_out = total;
        if (launches >= limit) return fail(CB_ENOTCONVERGED, "batch made no progress");
        return CB_OK;
    }

   private:
    std::unique_ptr<Pool<T>> pool;
    std::vector<std::unique_ptr<Stepper<T>>> items;
    std::vector<std::pair<int, int>> where;
    void* flush_buf = nullptr;
    long long flush_size = 0;
};

// ---------------------------------------------------------------- server
// Device memory of the served pool: one region reserved before the trace starts,
// carved into instance arenas first-fit, with freed blocks merged with their free
// neighbours, so admitting a request allocates nothing from the driver.
class ArenaRegion {
   public:
    ~ArenaRegion() { cudaFree(base); }
    int init(size_t bytes) {
        size = bytes & ~(size_t)255;
        if (cudaMalloc(&base, size) != cudaSuccess) {
            cudaGetLastError();
            return fail(CB_ENOMEM, "served pool: cudaMalloc of its %zu-byte region failed", size);
        }
        free_[0] = size;
        return CB_OK;
    }
    void* take(size_t n) {
        n = (n + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            const size_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > n) free_[off + n] = len - n;
            return static_cast<char*>(base) + off;
        }
        return nullptr;
    }
    void give(void* ptr, size_t n) {
        n = (n + 255) & ~(size_t)255;
        size_t off = static_cast<size_t>(static_cast<char*>(ptr) - static_cast<char*>(base));
        auto nx = free_.lower_bound(off);
        if (nx != free_.end() && off + n == nx->first) {  // merge with the block after
            n += nx->second;
            nx = free_.erase(nx);
        }
        if (nx != free_.begin()) {  // and with the block before
            auto pv = std::prev(nx);
            if (pv->first + pv->second == off) {
                pv->second += n;
                return;
            }
        }
        free_[off] = n;
    }
    size_t bytes() const { return size; }

   private:
    void* base = nullptr;
    size_t size = 0;
    std::map<size_t, size_t> free_;  // offset -> length
};

// One size class of the server: its slot table, its own attempt graph and stream,
// so each class advances at its own pace (a 32^3 request is not paced by a 256^3
// one), and its per-slot summaries copied back to pinned host memory.
template <class T> struct ServeClass {
    int nx = 0, nz = 0, method = 0, accurate = 0, split = 0, curv = 0, cap = 0, ntiles = 0, quantum = 1;
    long long bytes = 0;
    InstT<T>* table = nullptr;   // device slot table
    InstT<T>* h_table = nullptr; // pinned mirror, the source of the table's copies
    SlotSummary* d_sum = nullptr;
    SlotSummary* h_sum = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    cudaGraphExec_t g = nullptr;
    std::vector<int> slot_act;  // index into the active list, -1 for a free slot
    int active = 0;
    bool inflight = false;
};

template <class T> struct Active {
    std::unique_ptr<Stepper<T>> st;
    void* mem = nullptr;
    int req = -1, cls = -1, slot = -1;
    long long bytes = 0;
    double cancel_at = 0.0;  // > 0: trace time at which the request is cancelled
};

template <class T> struct Server {
    std::vector<ServeClass<T>> cls;
    ArenaRegion region;
    cudaStream_t adm = nullptr;  // admission / retirement stream (set-up of admitted instances)
    Ctrl* dummy_ctrl = nullptr;
    InstT<T> dummy{};
    double* stage = nullptr;     // phi0 of an admitted request

    ~Server() {
        for (auto& c : cls) {
            if (c.s) cudaStreamSynchronize(c.s);
            if (c.g) cudaGraphExecDestroy(c.g);
            cudaFree(c.table);
            cudaFree(c.d_sum);
            cudaFreeHost(c.h_table);
            cudaFreeHost(c.h_sum);
            if (c.ev) cudaEventDestroy(c.ev);
            if (c.s) cudaStreamDestroy(c.s);
        }
        if (adm) cudaStreamSynchronize(adm);
        cudaFree(dummy_ctrl);
        cudaFree(stage);
        if (adm) cudaStreamDestroy(adm);
    }

    int find(const Eff& e) const {
        for (size_t i = 0; i < cls.size(); ++i) {
            const auto& c = cls[i];
            if (c.nx == e.p.nx && c.nz == e.p.nz && c.method == e.p.method && c.accurate == e.accurate &&
                c.split == e.p.split && c.curv == e.p.curv)
                return (int)i;
        }
        return -1;
    }

    // classes, their graphs and every allocation of the trace, before it starts
    int setup(const cb_request* reqs, int n, long long budget, int max_slots, int quantum) {
        CB_CK(cudaStreamCreateWithFlags(&adm, cudaStreamNonBlocking));
        CB_CK(cudaMalloc(&dummy_ctrl, sizeof(Ctrl)));
        Ctrl dc;
        memset(&dc, 0, sizeof dc);
        dc.done = 1;
        CB_CK(cudaMemcpy(dummy_ctrl, &dc, sizeof dc, cudaMemcpyHostToDevice));
        memset(&dummy, 0, sizeof dummy);
        dummy.ctrl = dummy_ctrl;
        long long maxN = 0;
        std::vector<Eff> effs(n);
        for (int i = 0; i < n; ++i) {
            int rc = make_params(reqs[i].params, effs[i]);
            if (rc) return rc;
        }
        auto same_class = [](const Eff& a, const Eff& b) {
            return a.p.nx == b.p.nx && a.p.nz == b.p.nz && a.p.method == b.p.method && a.accurate == b.accurate &&
                   a.p.split == b.p.split && a.p.curv == b.p.curv;
        };
        for (int i = 0; i < n; ++i) {
            const Eff& e = effs[i];
            if (!Launch<T>::xy_supported(e.p.nx) || !Launch<T>::z_supported(e.p.nz))
                return fail(CB_EUNSUPPORTED, "request %d: grid %d^2x%d not built", i, e.p.nx, e.p.nz);
            maxN = std::max<long long>(maxN, e.p.N);
            if (find(e) >= 0) continue;
            // the trace's requests of this class: no more slots than that, since every
            // launch of the class graph runs (empty) CTAs for its free slots too
            int members = 0;
            for (int j = i; j < n; ++j) members += same_class(e, effs[j]) ? 1 : 0;
            ServeClass<T> c;
            c.nx = e.p.nx; c.nz = e.p.nz; c.method = e.p.method; c.accurate = e.accurate; c.split = e.p.split;
            c.curv = e.p.curv;
            c.bytes = (long long)instance_arena_bytes<T>(e.p);
            if (c.bytes > budget) return fail(CB_ENOMEM, "request %d needs %lld bytes, over the budget", i, c.bytes);
            c.cap = (int)std::max<long long>(1, std::min<long long>({(long long)max_slots, budget / c.bytes,
                                                                     (long long)members}));
            const int tx = Launch<T>::z_tile();
            c.ntiles = (e.p.ny * e.p.nc + tx - 1) / tx;
            // attempts per launch batch: more for small grids, whose attempts are short
            // next to a host round trip
            const double vol = (double)e.p.N / (128.0 * 128.0 * 128.0);
            c.quantum = (int)std::min(32.0 * quantum, std::max((double)quantum, quantum / std::max(vol, 1e-9)));
            c.slot_act.assign(c.cap, -1);
            CB_CK(cudaMalloc(&c.table, sizeof(InstT<T>) * c.cap));
            CB_CK(cudaMalloc(&c.d_sum, sizeof(SlotSummary) * c.cap));
            CB_CK(cudaMallocHost(&c.h_table, sizeof(InstT<T>) * c.cap));
            CB_CK(cudaMallocHost(&c.h_sum, sizeof(SlotSummary) * c.cap));
            for (int k = 0; k < c.cap; ++k) c.h_table[k] = dummy;
            CB_CK(cudaMemcpy(c.table, c.h_table, sizeof(InstT<T>) * c.cap, cudaMemcpyHostToDevice));
            CB_CK(cudaEventCreateWithFlags(&c.ev, cudaEventDisableTiming));
            // the twiddle tables of the class, made (and cached) now rather than at admission
            cudaError_t te = cudaSuccess;
            if (!twiddle_table<T>(e.p.nx, 1, &te) || !twiddle_table<T>(e.p.ny, 0, &te) ||
                !twiddle_table<T>(e.p.nz, 0, &te))
                return fail(CB_ECUDA, "twiddles: %s", cudaGetErrorString(te));
            if (sizeof(T) == 4 && (!twiddle_table<double>(e.p.nx, 1, &te) || !twiddle_table<double>(e.p.ny, 0, &te) ||
                                   !twiddle_table<double>(e.p.nz, 0, &te)))
                return fail(CB_ECUDA, "twiddles: %s", cudaGetErrorString(te));
            cls.push_back(c);
        }
        // Stream priorities by grid size: the device hands free SMs to the CTAs of the
        // smaller grids first, so their short attempts are not queued behind the large
        // grids' long launches (shortest job first across classes).
        int lo = 0, hi = 0;
        CB_CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        std::vector<long long> sizes;
        for (auto& c : cls) sizes.push_back((long long)c.nx * c.nx * c.nz);
        std::sort(sizes.begin(), sizes.end());
        sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
        const int levels = lo - hi + 1;  // hi is the numerically smallest (greatest) priority
        for (auto& c : cls) {
            const long long sz = (long long)c.nx * c.nx * c.nz;
            const int rank = (int)(std::lower_bound(sizes.begin(), sizes.end(), sz) - sizes.begin());
            const int pri = hi + (int)((long long)rank * levels / (long long)sizes.size());
            CB_CK(cudaStreamCreateWithPriority(&c.s, cudaStreamNonBlocking, std::min(pri, lo)));
            cudaGraph_t gr = nullptr;
            CB_CK(cudaStreamBeginCapture(c.s, cudaStreamCaptureModeThreadLocal));
            cudaError_t r = enqueue_group<T>(c.method, c.nx, c.nz, c.table, c.cap, c.ntiles, c.accurate, false,
                                             c.split, c.curv, c.s);
            cudaError_t ee = cudaStreamEndCapture(c.s, &gr);
            if (r != cudaSuccess || ee != cudaSuccess) {
                if (gr) cudaGraphDestroy(gr);
                return fail(CB_ECUDA, "class capture: %s", cudaGetErrorString(r != cudaSuccess ? r : ee));
            }
            cudaError_t ie = cudaGraphInstantiate(&c.g, gr, 0);
            cudaGraphDestroy(gr);
            CB_CK(ie);
        }
        size_t fr = 0, tot = 0;
        CB_CK(cudaMemGetInfo(&fr, &tot));
        const size_t margin = (size_t)2 << 30;
        size_t want = (size_t)budget;
        if (fr > margin) want = std::min(want, fr - margin);
        int rc = region.init(want);
        if (rc) return rc;
        for (auto& c : cls)
            if ((size_t)c.bytes > region.bytes())
                return fail(CB_ENOMEM, "a %d^2x%d instance needs %lld bytes, more than the %zu the device can reserve",
                            c.nx, c.nz, c.bytes, region.bytes());
        CB_CK(cudaMalloc(&stage, (size_t)maxN * sizeof(double)));
        return CB_OK;
    }

    // set up request r in a free slot of class ci on caller-owned memory; false when the
    // region has no block for it right now
    int admit(const cb_request& r, int ci, Active<T>& a, bool* placed) {
        ServeClass<T>& c = cls[ci];
        *placed = false;
        void* mem = region.take((size_t)c.bytes);
        if (!mem) return CB_OK;
        a.mem = mem;
        a.bytes = c.bytes;
        a.st.reset(new Stepper<T>());
        int rc = a.st->init_in(r.params, mem, adm);
        if (rc) return rc;
        const Params& p = a.st->params();
        const double L = (r.params.lenx > 0 ? r.params.lenx : 1.0) * kTwoPi;
        ellipsoid_kernel<<<1024, 256, 0, adm>>>(stage, p.nx, p.nz, L, p.eps, r.axes[0], r.axes[1], r.axes[2],
                                                r.centre[0], r.centre[1], r.centre[2], r.axes2[0], r.axes2[1],
                                                r.axes2[2], r.centre2[0], r.centre2[1], r.centre2[2]);
        CB_CK(cudaGetLastError());
        rc = a.st->set_phi(stage, true);  // ordered after the kernel on the same stream; synchronises it
        if (rc) return rc;
        rc = a.st->prepare_run(r.max_steps > 0 ? r.max_steps : INT_MAX / 2);
        if (rc) return rc;
        int k = 0;
        while (c.slot_act[k] >= 0) ++k;
        a.cls = ci;
        a.slot = k;
        c.h_table[k] = a.st->inst();
        // stream-ordered on the class stream: the slot changes between two of its batches
        CB_CK(cudaMemcpyAsync(c.table + k, c.h_table + k, sizeof(InstT<T>), cudaMemcpyHostToDevice, c.s));
        *placed = true;
        return CB_OK;
    }

    // empty the slot (stream-ordered) and give the arena back; the class is idle
    int retire(Active<T>& a) {
        ServeClass<T>& c = cls[a.cls];
        c.h_table[a.slot] = dummy;
        CB_CK(cudaMemcpyAsync(c.table + a.slot, c.h_table + a.slot, sizeof(InstT<T>), cudaMemcpyHostToDevice, c.s));
        CB_CK(cudaStreamSynchronize(c.s));
        c.slot_act[a.slot] = -1;
        c.active--;
        a.st.reset();  // synchronises the admission stream; the arena stays the region's
        region.give(a.mem, (size_t)a.bytes);
        a.mem = nullptr;
        return CB_OK;
    }

    int launch(ServeClass<T>& c) {
        for (int i = 0; i < c.quantum; ++i) CB_CK(cudaGraphLaunch(c.g, c.s));
        gather_kernel<T><<<(c.cap + 127) / 128, 128, 0, c.s>>>(c.table, c.cap, c.d_sum);
        CB_CK(cudaGetLastError());
        CB_CK(cudaMemcpyAsync(c.h_sum, c.d_sum, sizeof(SlotSummary) * c.cap, cudaMemcpyDeviceToHost, c.s));
        CB_CK(cudaEventRecord(c.ev, c.s));
        c.inflight = true;
        return CB_OK;
    }
};

// Continuous batching over an arrival trace, in real time.  Arrivals join a queue;
// every pass admits, in arrival order, each queued request whose size class has a
// free slot (a request whose class is full is passed over, not waited on) while the
// HBM budget and the pool's region hold its instance; a request the budget cannot
// hold stops admission behind it, so large requests are not starved.  Each class
// runs batches of attempts on its own stream; a class whose batch has finished
// retires its finished (or cancelled) requests, takes new ones, and starts its next
// batch at once.  A request with cancel_ms > 0 is cancelled that long after its
// arrival: dropped from the queue, or retired from its slot after its class's
// current batch, with CB_DONE_CANCELLED and its memory returned.
template <class T>
static int serve_impl(const cb_request* reqs, int n, long long budget, int max_slots, int quantum, cb_result* res,
                      double** phi_out, cb_serve_stats* stats) {
    Server<T> sv;
    int rc = sv.setup(reqs, n, budget, max_slots, quantum);
    if (rc) return rc;
    std::vector<int> rcls(n);
    for (int i = 0; i < n; ++i) {
        Eff e;
        make_params(reqs[i].params, e);
        rcls[i] = sv.find(e);
    }
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    auto now = [&]() { return std::chrono::duration<double>(clk::now() - t0).count(); };
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return reqs[a].arrival_s < reqs[b].arrival_s; });
    auto cancel_time = [&](int i) { return reqs[i].cancel_ms > 0 ? reqs[i].arrival_s + 1e-3 * reqs[i].cancel_ms : 0.0; };
    size_t next = 0;
    std::deque<int> queue;
    std::vector<Active<T>> act;  // stable indices: finished entries are recycled through `spare`
    std::vector<int> spare;
    long long used = 0, peak = 0;
    int done = 0, launches = 0;
    double point_steps = 0.0;

    auto finish = [&](int ai, int status_override) -> int {
        Active<T>& a = act[ai];
        const int i = a.req;
        int status = 0;
        int r = a.st->finish_run(&status);
        if (r) return r;
        cb_scalars sc;
        a.st->scalars(&sc);
        res[i].finished_s = now();
        res[i].latency_s = res[i].finished_s - res[i].arrival_s;
        res[i].E = sc.E;
        res[i].V = sc.V;
        res[i].S = sc.S;
        res[i].steps = sc.steps;
        res[i].attempts = sc.attempts;
        res[i].status = status_override >= 0 ? status_override : status;
        point_steps += (double)a.st->params().N * sc.steps;
        if (phi_out && phi_out[i]) {
            r = a.st->get_phi(phi_out[i], false);
            if (r) return r;
        }
        r = sv.retire(a);
        if (r) return r;
        used -= a.bytes;
        a.req = -1;
        spare.push_back(ai);
        ++done;
        return CB_OK;
    };

    while (done < n) {
        const double tnow = now();
        while (next < order.size() && reqs[order[next]].arrival_s <= tnow) queue.push_back(order[next++]);
        // cancellations of queued requests
        for (auto it = queue.begin(); it != queue.end();) {
            const double ct = cancel_time(*it);
            if (ct > 0 && ct <= tnow) {
                res[*it].arrival_s = reqs[*it].arrival_s;
                res[*it].finished_s = tnow;
                res[*it].latency_s = tnow - reqs[*it].arrival_s;
                res[*it].status = ST_CANCELLED;
                ++done;
                it = queue.erase(it);
            } else {
                ++it;
            }
        }
        // finished batches: retire what is done or cancelled
        for (auto& c : sv.cls) {
            if (!c.inflight || cudaEventQuery(c.ev) == cudaErrorNotReady) continue;
            CB_CK(cudaEventSynchronize(c.ev));  // reports a failed batch
            c.inflight = false;
            for (int k = 0; k < c.cap; ++k) {
                const int ai = c.slot_act[k];
                if (ai < 0) continue;
                const double ct = act[ai].cancel_at;
                const bool cancelled = ct > 0 && ct <= now();
                if (!c.h_sum[k].done && !cancelled) continue;
                rc = finish(ai, c.h_sum[k].done ? -1 : ST_CANCELLED);
                if (rc) return rc;
            }
        }
        // admission: arrival order; full classes are passed over, the budget stops it
        for (auto it = queue.begin(); it != queue.end();) {
            const int i = *it;
            ServeClass<T>& c = sv.cls[rcls[i]];
            if (c.inflight || c.active >= c.cap) { ++it; continue; }
            if (used + c.bytes > budget) break;
            int ai;
            if (!spare.empty()) { ai = spare.back(); spare.pop_back(); }
            else { ai = (int)act.size(); act.emplace_back(); }
            bool placed = false;
            rc = sv.admit(reqs[i], rcls[i], act[ai], &placed);
            if (rc) return rc;
            if (!placed) { spare.push_back(ai); break; }  // the region is fragmented or full
            Active<T>& a = act[ai];
            a.req = i;
            a.cancel_at = cancel_time(i);
            c.slot_act[a.slot] = ai;
            c.active++;
            used += a.bytes;
            peak = std::max(peak, used);
            res[i].arrival_s = reqs[i].arrival_s;
            res[i].admitted_s = now();
            res[i].bytes = a.bytes;
            it = queue.erase(it);
        }
        // every idle class with work starts its next batch
        bool any = false;
        for (auto& c : sv.cls) {
            if (!c.inflight && c.active > 0) {
                rc = sv.launch(c);
                if (rc) return rc;
                launches += c.quantum;
            }
            any = any || c.inflight;
        }
        if (!any) {
            if (next < order.size()) {
                const double wait = reqs[order[next]].arrival_s - now();
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
            }
            continue;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    if (stats) {
        stats->wall_s = now();
        stats->completed = done;
        stats->point_steps = point_steps;
        stats->graph_launches = launches;
        stats->peak_bytes = peak;
    }
    return CB_OK;
}

}  // namespace cb

// ====================================================================== C ABI
struct cb_batch {
    std::unique_ptr<cb::BatchBase> impl;
};

extern "C" {

int cb_batch_create(const cb_params* ps, int n, cb_batch** out) { return cb_batch_create_ex(ps, n, 0, out); }

int cb_batch_create_ex(const cb_params* ps, int n, int flags, cb_batch** out) {
    if (!ps || n <= 0 || !out) return cb::fail(CB_EINVAL, "bad batch arguments");
    if (flags & ~CB_BATCH_PERSISTENT) return cb::fail(CB_EINVAL, "unknown batch flags %d", flags);
    const bool persistent = (flags & CB_BATCH_PERSISTENT) != 0;
    *out = nullptr;
    for (int i = 1; i < n; ++i)
        if (ps[i].precision != ps[0].precision) return cb::fail(CB_EINVAL, "a batch holds one precision");
    std::unique_ptr<cb_batch> b(new cb_batch);
    int rc;
    if (ps[0].precision == CB_FP32) {
        auto* p = new cb::Batch<float>();
        b->impl.reset(p);
        rc = p->init(ps, n, persistent);
    } else {
        auto* p = new cb::Batch<double>();
        b->impl.reset(p);
        rc = p->init(ps, n, persistent);
    }
    if (rc) return rc;
    *out = b.release();
    return CB_OK;
}

int cb_batch_destroy(cb_batch* b) {
    delete b;
    return CB_OK;
}

#define CB_B(b, i) \
    if (!(b) || !(b)->impl || (i) < 0 || (i) >= (b)->impl->size()) return cb::fail(CB_EINVAL, "bad batch index")

int cb_batch_set_phi(cb_batch* b, int i, const double* phi, int on_device) {
    CB_B(b, i);
    return b->impl->set_phi(i, phi, on_device != 0);
}
int cb_batch_get_phi(cb_batch* b, int i, double* phi, int on_device) {
    CB_B(b, i);
    return b->impl->get_phi(i, phi, on_device != 0);
}
int cb_batch_scalars(cb_batch* b, int i, cb_scalars* s) {
    CB_B(b, i);
    return b->impl->scalars(i, s);
}
int cb_batch_run(cb_batch* b, int nsteps, cb_run_stats* st) {
    CB_B(b, 0);
    return b->impl->run(nsteps, st, 0, nullptr);
}
int cb_batch_run_timed(cb_batch* b, int nsteps, long long flush_bytes, double* device_ms, cb_run_stats* st) {
    CB_B(b, 0);
    return b->impl->run(nsteps, st, flush_bytes, device_ms);
}

int cb_serve_trace(const cb_request* reqs, int n, long long hbm_budget_bytes, int max_slots_per_class, int quantum,
                   cb_result* results, double** phi_out, cb_serve_stats* stats) {
    if (!reqs || n <= 0 || !results || hbm_budget_bytes <= 0) return cb::fail(CB_EINVAL, "bad serve arguments");
    memset(results, 0, sizeof(cb_result) * (size_t)n);
    for (int i = 1; i < n; ++i)
        if (reqs[i].params.precision != reqs[0].params.precision)
            return cb::fail(CB_EINVAL, "a trace holds one precision");
    const int q = quantum > 0 ? quantum : 4;
    const int ms = max_slots_per_class > 0 ? max_slots_per_class : 64;
    if (reqs[0].params.precision == CB_FP32)
        return cb::serve_impl<float>(reqs, n, hbm_budget_bytes, ms, q, results, phi_out, stats);
    return cb::serve_impl<double>(reqs, n, hbm_budget_bytes, ms, q, results, phi_out, stats);
}

}  // extern "C"
