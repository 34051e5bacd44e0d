// The persistent batched attempt (FP32 form, ETD-RK2): one launch of two-CTA clusters
// runs one attempt of every instance of a batched pool by walking the work list of
// mega.h.  The units run the same pass bodies as the one-pass kernels (z_body,
// xyc_body, xy_body, prologue_body with PDL = false) on 512-thread CTAs: z tiles and
// planes below 64^2 on thread groups of the one-pass kernels' shapes (two 16-column,
// 256-thread z tiles a CTA; two 256-thread or four 128-thread planes), each group on its
// own named barrier and slice of shared memory; planes from 64^2 on both CTAs of the
// cluster (512 threads a CTA; the one-pass kernel takes 256 at 64^2).  Each instance
// keeps its own dt and decision, so its result does not depend on the other instances of
// the pool; it is bitwise that of the per-class graph except for 64^2 planes, whose sums
// differ in summation order.
//
// Hand-over: rank 0 of a cluster claims the next unit from the shared counter as the
// current one starts, and its descriptor streams into shared memory (cp.async) under the
// current unit's work.  Between units rank 0 checks the next unit's dependency, leaves
// the unit and its descriptor in one of two slots of its shared memory, and a cluster
// barrier hands them to rank 1 (which copies them through distributed shared memory).
// Both CTAs run the same sequence of units and meet the same cluster barriers inside the
// cluster xy body.  The instance pointers sit in shared memory from the start.
//
// Completion: after a unit, warp 1 of each CTA counts it in its instance's phase counter
// behind a release fence (beside rank 0's preparation of the next hand-over), and the CTA
// that completes an instance's candidate phase runs the instance's decision.
//
// Waits: rank 0's thread 0 polls the previous phase's completion counter of the unit's
// instance with a bounded number of polls, then acquires; the cluster barrier passes that
// on to rank 1.  A wait that runs out counts in err and the unit runs anyway (its results
// are then not used: the pool reports the attempt as failed), so the control flow of the
// two CTAs of a cluster never parts.
#pragma once
#include <cooperative_groups.h>

#include <cstddef>

#include "mega.h"
#include "misc_kernels.cuh"
#include "xy_cluster.cuh"
#include "xy_kernel.cuh"
#include "z_kernel.cuh"

namespace cb {

// the unit bodies are separate functions (their registers are allocated one by one)
#if defined(CB_EMULATION)
#define CB_NOINLINE __attribute__((noinline))
#else
#define CB_NOINLINE __noinline__
#endif

// the grid edges the kernel is built for (each adds a z body and an xy body)
#ifndef CB_MEGA_SIZES
#define CB_MEGA_SIZES(X) X(32) X(48) X(64) X(96) X(128)
#endif
// polls of a dependency counter before the wait is given up (64-ns sleeps and an L2
// load each: ~0.1 s, some hundred times a unit's longest legitimate wait)
#ifndef CB_MEGA_SPIN
#define CB_MEGA_SPIN (1 << 20)
#endif

__host__ __device__ constexpr size_t mega_align(size_t b) { return (b + 15) & ~(size_t)15; }

// the head of a CTA's dynamic shared memory
struct MegaSlot {
    unsigned t;  // the unit (>= ntasks: the walk is over)
    int pad[3];
    MegaTask task;
};
struct MegaHeadLayout {
    MegaSlot slot[2];  // rank 0's hand-over slots (round parity)
    MegaSlot cur;      // this CTA's unit of the round
    MegaTask next;     // rank 0: the next unit's descriptor, streamed in under the current unit
    int last;          // the prologue's last-block flag
    int pad;
    ProState pro;      // the prologue's block state
    const InstT<float>* insts[kMegaInstCache];
};
static_assert(sizeof(MegaHeadLayout) <= kMegaHead, "the head fits");
static_assert(offsetof(MegaHeadLayout, next) % 16 == 0, "cp.async target aligned");

// a 16-byte global -> shared copy that completes asynchronously (this thread waits for it
// with mega_copy_wait)
__device__ __forceinline__ void mega_copy16(void* dst, const void* src) {
#if defined(__CUDA_ARCH__)
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n\tcp.async.commit_group;" ::"r"(d), "l"(src) : "memory");
#else
    memcpy(dst, src, 16);
#endif
}
__device__ __forceinline__ void mega_copy_wait() {
#if defined(__CUDA_ARCH__)
    asm volatile("cp.async.wait_all;" ::: "memory");
#endif
}

// z tile `tile` on thread group j of the CTA (256 threads, its own slice of shared memory)
template <int N>
__device__ CB_NOINLINE void mega_z(const InstT<float>& I, int tile, int mode, unsigned char* sm, int j) {
    ZArgs za = {};
    za.mode = mode;
    za.role = mode == Z_ETD2_S1 ? R_WORK : R_CAND;
    const Grp g{1 + j, kMegaZThreads, (int)threadIdx.x - j * kMegaZThreads};
    constexpr size_t bytes = mega_align(z_smem_bytes<float, N, kMegaZTX>());
    z_body<float, N, kMegaZTX, kMegaZThreads, ZG_ETD2, 0, false>(I, tile, za, sm + j * bytes, g);
}

// plane `plane` on the cluster (from 64^2), or on thread group j of the CTA
template <int N>
__device__ CB_NOINLINE void mega_xy(const InstT<float>& I, int plane, int role, unsigned char* sm, int j) {
    XYArgs xa = {};
    xa.mode = XY_FUSED;
    xa.role = role;
    if constexpr (mega_cluster_xy(N)) {
        xyc_body<float, N, kMegaThreads, 0, false>(I, plane, xa, sm);
    } else {
        constexpr int NT = mega_xy_threads(N);
        const Grp g{1 + j, NT, (int)threadIdx.x - j * NT};
        constexpr size_t bytes = mega_align(xy_smem_bytes<float, N>(2));
        xy_body<float, N, NT, 2, 0, false>(I, plane, xa, sm + j * bytes, g);
    }
}

__device__ CB_NOINLINE void mega_pro(const InstT<float>& I, int blk, int nblk, int accurate, MegaHeadLayout* h) {
    prologue_body<float>(I, blk, nblk, accurate, 0, &h->pro, &h->last);
}

__device__ CB_NOINLINE void mega_decide(const InstT<float>& I) { decide_one(I, 0); }

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kMegaThreads, 2) mega_kernel(const MegaArgs a) {
    namespace cg = cooperative_groups;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int tid = threadIdx.x;
    MegaHeadLayout* h = reinterpret_cast<MegaHeadLayout*>(smem_raw);
    const MegaSlot* src = rank == 0 ? h->slot : cl.map_shared_rank(h->slot, 0);
    unsigned char* sm = smem_raw + kMegaHead;
    const int ncache = a.ninst < kMegaInstCache ? a.ninst : kMegaInstCache;
    for (int i = tid; i < ncache; i += kMegaThreads) h->insts[i] = a.insts[i];
    unsigned claimed = 0;  // rank 0, thread 0: the unit of the next round
    if (rank == 0 && tid == 0) {
        claimed = atomicAdd(a.ticket, 1u);
        if (claimed < (unsigned)a.ntasks) h->next = a.tasks[claimed];
    }
    for (int round = 0;; ++round) {
        if (rank == 0 && tid == 0) {
            // the round's unit, its descriptor and its dependency, checked before the hand-over
            MegaSlot& s = h->slot[round & 1];
            s.t = claimed;
            if (claimed < (unsigned)a.ntasks) {
                mega_copy_wait();
                s.task = h->next;
                if (s.task.phase != MP_PRO) {
                    const int dep = s.task.inst * MP_N + s.task.phase - 1;
                    const volatile unsigned* d = a.done + dep;
                    const volatile unsigned* failed = a.err;
                    const unsigned need = a.need[dep];
                    int n = 0;
                    // once any wait of the launch has run out, none waits: the attempt is void
                    // and ends without a further bound's delay per unit
                    while (*d < need && *failed == 0u) {
                        if (++n > CB_MEGA_SPIN) {
                            atomicAdd(a.err, 1u);
                            break;
                        }
                        __nanosleep(64);
                    }
                    CB_FENCE();  // the previous phase's writes before this unit's reads
                }
            }
        }
        // the round's unit is in rank 0's slot, its dependency met; both CTAs are done with
        // the last round.  The barrier's release / acquire passes rank 0's acquisition of the
        // previous phase's writes on to rank 1.
        cl.sync();
        if (tid == 0) h->cur = src[round & 1];
        __syncthreads();
        const unsigned t = h->cur.t;
        if (t >= (unsigned)a.ntasks) break;
        const MegaTask task = h->cur.task;
        if (rank == 0 && tid == 0) {  // claim the next unit and stream its descriptor in
            claimed = atomicAdd(a.ticket, 1u);
            if (claimed < (unsigned)a.ntasks) mega_copy16(&h->next, a.tasks + claimed);
        }
        const int slot = task.inst * MP_N + task.phase;
        const InstT<float>& I = task.inst < ncache ? *h->insts[task.inst] : *a.insts[task.inst];
        const int n = task.size & 0xffff;
        const int part = 2 * task.unit + rank;
        switch (task.phase) {
            case MP_PRO:
                mega_pro(I, part, (int)a.need[slot], task.size >> 16, h);
                break;
            case MP_Z1:
            case MP_Z2: {
                const int mode = task.phase == MP_Z1 ? Z_ETD2_S1 : Z_ETD2_S2;
                constexpr int G = kMegaThreads / kMegaZThreads;
                const int j = tid / kMegaZThreads;
                switch (n) {
#define CASE(N) case N: mega_z<N>(I, part * G + j, mode, sm, j); break;
                    CB_MEGA_SIZES(CASE)
#undef CASE
                    default: break;
                }
                break;
            }
            default: {  // MP_XYW, MP_XYC
                const int role = task.phase == MP_XYW ? R_WORK : R_CAND;
                const int G = kMegaThreads / mega_xy_threads(n);
                const int j = mega_cluster_xy(n) ? 0 : tid / mega_xy_threads(n);
                const int plane = mega_cluster_xy(n) ? task.unit : part * G + j;
                switch (n) {
#define CASE(N) case N: mega_xy<N>(I, plane, role, sm, j); break;
                    CB_MEGA_SIZES(CASE)
#undef CASE
                    default: break;
                }
                break;
            }
        }
        __syncthreads();
        // the completion count from warp 1, so that its fence (which waits for this unit's
        // stores) runs beside rank 0's thread 0 preparing the next hand-over
        if (tid == 32) {
            CB_FENCE();  // this CTA's writes before its completion count
            const unsigned prev = atomicAdd(a.done + slot, 1u);
            if (task.phase == MP_XYC && prev + 1 == a.need[slot]) {
                CB_FENCE();  // every CTA of the phase has counted: their sums are final
                mega_decide(I);
            }
        }
    }
    cl.sync();  // neither CTA leaves while its partner may read its slots
}

}  // namespace cb
