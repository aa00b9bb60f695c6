// Grid-wide barrier of the persistent step kernels, with a bounded wait.
//
// The kernels are launched cooperatively (every block resident at once), so a
// barrier over all blocks cannot deadlock by itself; the wait is still bounded
// so that a fault elsewhere can never leave the GPU spinning: a block that
// waits longer than `limit_ns` (device global timer) sets `status` and
// returns, and every block that later reaches a barrier (or starts) sees the
// status and returns too.  The host reads `status` after the launch.
//
// Protocol: one 64-bit arrival counter that only grows.  Thread 0 of each
// block adds 1 with release semantics (after a block barrier, so the block's
// writes are published with it) and then polls the counter with acquire
// loads until it reaches the arrivals of this barrier, (k + 1) x expected for
// the k-th barrier since the counter was zeroed; a block barrier then lets the
// block's other threads go on (the acquire also makes the other blocks' writes
// visible to their ordinary loads).  No reset, no second word: the critical
// path is one atomic and one poll.  The counter is zeroed by the host before
// each run; a block carries the value it expects next.
#pragma once

#include <cuda_runtime.h>

namespace sihg {

struct GridBar {
    unsigned long long* count;   // [1] arrivals since the host zeroed it
    int* status;                 // [1] 0 ok, 1 a wait ran out
    unsigned expected;           // blocks that arrive at every barrier (the grid)
    unsigned long long limit_ns; // longest wait of one barrier
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long add_release_u64(unsigned long long* p, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.release.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}

__device__ __forceinline__ int ld_status(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Arrivals already counted when the kernel starts, rounded down to whole
// barriers (every block reads a value below the first barrier's target: that
// barrier cannot complete before all blocks arrived).
__device__ __forceinline__ unsigned long long grid_start(const GridBar& g) {
    const unsigned long long c = ld_acquire_u64(g.count);
    return c - c % g.expected;
}

// All blocks of the grid; returns false (uniformly within the block) when a
// wait ran out here or elsewhere; the caller then returns.  `next` holds the
// counter value this block waits for at its next barrier minus `expected`.
__device__ __forceinline__ bool grid_barrier(const GridBar& g, unsigned long long& base) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        const unsigned long long target = base + g.expected;
        add_release_u64(g.count, 1ull);
        const unsigned long long t0 = global_ns();
        unsigned spins = 0;
        while (ld_acquire_u64(g.count) < target) {
            if ((++spins & 31u) == 0u) {
                if (ld_status(g.status) != 0) {
                    good = 0;
                    break;
                }
                if (global_ns() - t0 > g.limit_ns) {
                    atomicExch(g.status, 1);
                    good = 0;
                    break;
                }
            }
        }
        base = target;
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

}  // namespace sihg
