// Test infrastructure: the emulated launch of tests/emu (one OS thread per CUDA thread of
// a cluster, clusters of a grid one after another), shared by the emulation drivers
// attempt.cpp and mega_attempt.cpp.  Include once per program, after cuda_runtime.h.
#pragma once
#include <functional>
#include <thread>
#include <vector>

#include "cuda_runtime.h"

namespace emu {
thread_local Block* t_blk = nullptr;
thread_local dim3 t_tid, t_bid;
dim3 g_bdim, g_gdim;
std::mutex g_atomic_mu;

// body() for every thread of the grid, `clus` consecutive blocks (along x) at a time;
// one OS thread per CUDA thread of a cluster, reused for every cluster of the grid
void launch(dim3 grid, int nt, size_t smem, int clus, const std::function<void()>& body) {
    g_bdim = dim3(nt);
    g_gdim = grid;
    const int total = nt * clus;
    Cluster cl;
    std::vector<Block> blocks(clus);
    for (int r = 0; r < clus; ++r) {
        blocks[r].ex = new double[nt];
        blocks[r].smem = (unsigned char*)malloc(smem ? smem : 1);
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
        free(b.smem);
        delete[] b.ex;
    }
}
}  // namespace emu
