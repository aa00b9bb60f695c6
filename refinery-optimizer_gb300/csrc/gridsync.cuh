// Grid-wide barrier of the persistent step kernel, with a bounded wait.
//
// The kernel is launched cooperatively (every block resident at once), so a
// barrier over all blocks cannot deadlock by itself; the wait is still bounded
// so that a fault elsewhere can never leave the GPU spinning: a block that
// waits longer than `limit_ns` (device global timer) sets `status` and
// returns, and every block that later reaches a barrier (or starts) sees the
// status and returns too.  The host reads `status` after the launch.
//
// Protocol: thread 0 of each block publishes its block's writes (fence),
// counts itself in `arrive`; the last arriver resets `arrive` and then
// advances `gen` with a release store; the others poll `gen` with acquire
// loads.  The fence after the wait makes the other blocks' writes visible to
// this block's ordinary loads (L1 included); a block barrier then releases the
// block.  `gen` only grows, and no block can start barrier k + 1 before
// barrier k completed, so each block can carry the value it expects.
#pragma once

#include <cuda_runtime.h>

namespace sihg {

struct GridBar {
    unsigned* arrive;            // [1] arrivals at the current barrier
    unsigned* gen;               // [1] completed barriers
    int* status;                 // [1] 0 ok, 1 a wait ran out
    unsigned expected;           // blocks that arrive at every barrier (the grid)
    unsigned long long limit_ns; // longest wait of one barrier
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_status(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Value of `gen` when the kernel starts (every block reads the same value: the
// first barrier cannot complete before all blocks arrived).
__device__ __forceinline__ unsigned grid_gen(const GridBar& g) { return ld_acquire_u32(g.gen); }

// All blocks of the grid; returns false (uniformly within the block) when a
// wait ran out here or elsewhere; the caller then returns.
__device__ __forceinline__ bool grid_barrier(const GridBar& g, unsigned& gen) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        const unsigned target = gen + 1u;
        __threadfence();
        if (atomicAdd(g.arrive, 1u) + 1u == g.expected) {
            *g.arrive = 0u;
            __threadfence();
            st_release_u32(g.gen, target);
        } else {
            const unsigned long long t0 = global_ns();
            unsigned spins = 0;
            while (ld_acquire_u32(g.gen) != target) {
                if (ld_status(g.status) != 0) {
                    good = 0;
                    break;
                }
                if ((++spins & 63u) == 0u && global_ns() - t0 > g.limit_ns) {
                    atomicExch(g.status, 1);
                    good = 0;
                    break;
                }
                if (spins > 256u) __nanosleep(64);
            }
        }
        __threadfence();
        gen = target;
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

}  // namespace sihg
