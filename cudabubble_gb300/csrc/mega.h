// Persistent batched attempt (FP32 form, ETD-RK2): the work list and the arguments of
// the one kernel that runs one attempt of every instance of a batched pool
// (mega.cuh), shared by the host side (pool.cu) and the device side.
//
// An attempt of one instance is five phases, each a set of units:
//   MP_PRO  prologue and coefficient-table fill      (units of two 512-thread blocks)
//   MP_Z1   z pass, stage 1                          (units of four 16-column tiles, two a
//                                                     CTA on 256-thread groups)
//   MP_XYW  fused xy pass of the work stage           (a plane on both CTAs of a cluster
//                                                     from 64^2, else 4 or 8 planes on
//                                                     256- or 128-thread groups)
//   MP_Z2   z pass, stage 2                          (as MP_Z1)
//   MP_XYC  fused xy pass of the candidate, then the decision (the CTA that ends the
//           phase runs it)
// The work list holds every unit of every instance in phase-major order (largest grids
// first within a phase).  Persistent two-CTA clusters claim units in list order from
// one counter, so a unit waits only on units claimed before it and the walk cannot
// deadlock whatever number of clusters is resident.  A unit waits (bounded) until the
// counter of its instance's previous phase is complete.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "cb_inst.h"

namespace cb {

enum MegaPhase { MP_PRO = 0, MP_Z1 = 1, MP_XYW = 2, MP_Z2 = 3, MP_XYC = 4, MP_N = 5 };

struct MegaTask {
    int phase;  // MegaPhase
    int inst;   // index into MegaArgs::insts
    int unit;   // CTA rank r of the cluster runs part k = 2 unit + r: on the cluster xy pass
                // the plane `unit` itself; else its thread group j runs z tile or plane
                // k G + j of the G groups a CTA holds
    int size;   // grid edge of the phase's transform (nz for z, nx for xy); bit 16: the
                // class's accurate-coefficient mode
};

struct MegaArgs {
    const MegaTask* tasks;
    const InstT<float>* const* insts;  // table entries of the pool's classes
    const unsigned* need;              // [inst][MP_N] CTA completions that end each phase
    unsigned* done;                    // [inst][MP_N] completions of this attempt (zeroed before)
    unsigned* ticket;                  // next unclaimed unit (zeroed before)
    unsigned* err;                     // waits that ran out of their bound (0 when healthy)
    int ntasks;
    int ninst;                         // entries of insts
};

constexpr int kMegaThreads = 512;   // threads of every CTA
constexpr int kMegaZTX = 16;        // z tile: the one-pass kernel's 16 columns on 256 threads,
constexpr int kMegaZThreads = 256;  // two tiles side by side in a CTA
constexpr int kMegaInstCache = 256; // instance pointers a CTA keeps in shared memory
constexpr int kMegaHead = 2304;     // dynamic shared-memory bytes before the bodies' region
constexpr int kMegaProRows = 1024;  // coefficient-table entries per prologue unit (two blocks)

// planes of n^2 run on two-CTA clusters (both CTAs of a unit); smaller ones side by side
// in a CTA, each on the thread count of the one-pass kernel (128 threads to 32^2, else 256)
__host__ __device__ constexpr bool mega_cluster_xy(int n) { return n >= 64; }
__host__ __device__ constexpr int mega_xy_threads(int n) { return n <= 32 ? 128 : 256; }

// one size class of the pool: instances [first, first + cap) of the instance table
struct MegaClass {
    int nx, nz, accurate, cap, first;
};

// units of phase ph for one instance of class c
inline int mega_units(const MegaClass& c, int ph) {
    const int nc = c.nx / 2 + 1;
    const int kmax = 2 * (c.nx / 2) * (c.nx / 2) + (c.nz / 2) * (c.nz / 2);
    const int ztiles = (c.nx * nc + kMegaZTX - 1) / kMegaZTX;
    switch (ph) {
        case MP_PRO: return std::max(1, (kmax + 1 + kMegaProRows - 1) / kMegaProRows);
        case MP_Z1:
        case MP_Z2: {  // two CTAs of two tiles
            const int per = 2 * (kMegaThreads / kMegaZThreads);
            return (ztiles + per - 1) / per;
        }
        default: {  // a plane on the cluster, or two CTAs of side-by-side planes
            const int per = 2 * (kMegaThreads / mega_xy_threads(c.nx));
            return mega_cluster_xy(c.nx) ? c.nz : (c.nz + per - 1) / per;
        }
    }
}

// The work list of one attempt (phase-major, larger grids first within a phase) and the
// CTA completions that end each phase of each instance (need[inst * MP_N + phase]).
inline void mega_plan(const std::vector<MegaClass>& cls, std::vector<MegaTask>& tasks,
                      std::vector<unsigned>& need) {
    int ninst = 0;
    for (auto& c : cls) ninst = std::max(ninst, c.first + c.cap);
    need.assign((size_t)ninst * MP_N, 0u);
    tasks.clear();
    std::vector<int> order(cls.size());
    for (size_t i = 0; i < cls.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (long long)cls[a].nx * cls[a].nx * cls[a].nz > (long long)cls[b].nx * cls[b].nx * cls[b].nz;
    });
    for (int ph = 0; ph < MP_N; ++ph)
        for (int ci : order) {
            const MegaClass& c = cls[ci];
            const int u = mega_units(c, ph);
            const int size = ((ph == MP_Z1 || ph == MP_Z2) ? c.nz : c.nx) | (c.accurate ? 1 << 16 : 0);
            for (int k = 0; k < c.cap; ++k) {
                const int inst = c.first + k;
                need[(size_t)inst * MP_N + ph] = 2u * (unsigned)u;
                for (int j = 0; j < u; ++j) tasks.push_back(MegaTask{ph, inst, j, size});
            }
        }
}

bool mega_size_ok(int n);                 // n is a grid edge the kernel is built for
size_t mega_smem_bytes();                 // dynamic shared memory of one CTA
int mega_max_clusters();                  // two-CTA clusters resident at once (0: error)
cudaError_t mega_launch(const MegaArgs& a, int nclusters, cudaStream_t s);

}  // namespace cb
