// Test infrastructure: the cluster subset of cooperative groups for the host emulation
// (cuda_runtime.h beside this file); distributed shared memory maps to the partner block.
#pragma once
#include "cuda_runtime.h"
namespace cooperative_groups {
struct cluster_group {
    unsigned block_rank() const { return (unsigned)emu::t_blk->rank; }
    void sync() const { emu::t_blk->cl->bar.wait(); }
    template <class T> T* map_shared_rank(T* p, int r) const {
        emu::Block* me = emu::t_blk;
        emu::Block* other = me->cl->blocks[r];
        const size_t off = (size_t)((unsigned char*)p - me->smem);
        return (T*)(other->smem + off);
    }
};
inline cluster_group this_cluster() { return cluster_group{}; }
}  // namespace cooperative_groups
