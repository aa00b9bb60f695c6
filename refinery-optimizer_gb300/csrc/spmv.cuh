// Sparse matrix-vector core of the PDHG engine.
//
// A "segment matrix" is one side of the LP matrix: the rows of A (CSR, used
// for A x) or the columns of A (CSC, used for A^T y).  Entries are stored as
// packed 8-byte pairs {index, float bits}: one 64-bit load brings the index and
// the value of a nonzero.
//
// Memory-level parallelism is what bounds these kernels (two dependent loads
// per nonzero: the pair, then the gathered vector element), so every lane
// issues its loads in batches of U: U pair loads, then U gathers, then U FMAs,
// with out-of-range slots predicated off.  The next segment's pointers and the
// epilogue's own operands are loaded before the current dot product so their
// latency overlaps it.
//
// Work split of the grid-stride form (plain path):
//   * light segments (length <= heavy_threshold): groups of `lanes` threads,
//     natural segment order (the epilogue's vector accesses stay coalesced);
//   * heavy segments: listed in heavy_idx, one warp each, in the first
//     heavy_blocks blocks of the grid.
// The epilogue is a functor with
//     using Pre = ...;  Pre pre(int seg);  void apply(int seg, float dot, const Pre&);
// pre() loads the segment's operands, apply() performs the fused update.
//
// EXACT mode reproduces the reference kernels' arithmetic
// (core/src/gpu/cuda_pdhg.cu:14-49): one thread per segment, products and sums
// in entry order, no fused multiply-add.
#pragma once

#include "common.cuh"

namespace sihg {

struct SegMatrix {
    int nseg;          // segments (rows for CSR, columns for CSC)
    const int* ptr;    // [nseg + 1]
    const int2* pairs; // [nnz] {index, __float_as_int(value)}
};

struct SpmvPlan {
    int lanes;            // threads per light segment: 1, 2, 4, 8, 16 or 32
    int heavy_threshold;  // longer segments go to the heavy list
    int heavy_count;
    const int* heavy_idx; // [heavy_count] segment ids
    int heavy_blocks;     // leading blocks that process heavy segments
    int light_blocks;
    int threads;          // threads per block (multiple of 32)
    int grid() const { return heavy_blocks + light_blocks; }
};

constexpr int kBatch = 4;  // loads in flight per lane per batch

__device__ __forceinline__ int2 ld_pair(const int2* p) {
    int2 v;
    asm("ld.global.nc.L1::no_allocate.v2.s32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ float ld_vec(const float* p) { return __ldg(p); }

// This lane's share of a segment dot product: entries beg+lane0, +L, +2L, ...
__device__ __forceinline__ float seg_dot(const int2* __restrict__ pairs, int beg, int end, int lane0, int L,
                                         const float* __restrict__ vec) {
    float acc[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) acc[u] = 0.f;
    for (int k = beg + lane0; k < end; k += kBatch * L) {
        int2 p[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) p[u] = (k + u * L < end) ? ld_pair(pairs + k + u * L) : make_int2(0, 0);
        float v[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) v[u] = (k + u * L < end) ? ld_vec(vec + p[u].x) : 0.f;
#pragma unroll
        for (int u = 0; u < kBatch; ++u) acc[u] = fmaf(__int_as_float(p[u].y), v[u], acc[u]);
    }
    return (acc[0] + acc[1]) + (acc[2] + acc[3]);
}

// Compensated share (Ogita-Rump-Oishi Dot2): returns s and e with s + e equal
// to this lane's partial dot product evaluated in about twice FP32 precision.
__device__ __forceinline__ void seg_dot2(const int2* __restrict__ pairs, int beg, int end, int lane0, int L,
                                         const float* __restrict__ vec, float& s_out, float& e_out) {
    float s = 0.f, e = 0.f;
    for (int k = beg + lane0; k < end; k += kBatch * L) {
        int2 p[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) p[u] = (k + u * L < end) ? ld_pair(pairs + k + u * L) : make_int2(0, 0);
        float v[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) v[u] = (k + u * L < end) ? ld_vec(vec + p[u].x) : 0.f;
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
            float pr, pe, ss, se;
            two_prod(__int_as_float(p[u].y), v[u], pr, pe);
            two_sum(s, pr, ss, se);
            s = ss;
            e = __fadd_rn(e, __fadd_rn(pe, se));
        }
    }
    s_out = s;
    e_out = e;
}

// Reference-order dot: sum = sum + v * x, entry by entry, unfused.
__device__ __forceinline__ float seg_dot_exact(const int2* __restrict__ pairs, int beg, int end,
                                               const float* __restrict__ vec) {
    float s = 0.f;
    for (int k = beg; k < end; ++k) {
        const int2 p = ld_pair(pairs + k);
        s = __fadd_rn(s, __fmul_rn(__int_as_float(p.y), ld_vec(vec + p.x)));
    }
    return s;
}

// Sum over the L lanes of a group (lane 0 of the group gets the total).
__device__ __forceinline__ float group_sum(float s, int L) {
    for (int o = L >> 1; o > 0; o >>= 1) s += __shfl_down_sync(FULL_MASK, s, o, L);
    return s;
}

// Compensated group sum of (s, e) pairs.
__device__ __forceinline__ void group_sum2(float& s, float& e, int L) {
    for (int o = L >> 1; o > 0; o >>= 1) {
        const float s2 = __shfl_down_sync(FULL_MASK, s, o, L);
        const float e2 = __shfl_down_sync(FULL_MASK, e, o, L);
        float t, te;
        two_sum(s, s2, t, te);
        s = t;
        e = __fadd_rn(e, __fadd_rn(e2, te));
    }
}

// Light segments [s0, s1) handled by groups of L lanes; this thread's group is
// `group` of `ngroups` (group-strided).  Segments longer than `heavy_threshold`
// are skipped (handled elsewhere).  Warp-uniform loop.
template <bool EXACT, class Epi>
__device__ __forceinline__ void spmv_groups(const SegMatrix& A, const float* __restrict__ vec, int s0, int s1,
                                            int group, int ngroups, int L, int heavy_threshold, Epi& epi) {
    const int sub = (threadIdx.x & 31) & (L - 1);
    // first segment of this group; every lane of a warp runs the same trip count
    int r = s0 + group;
    const int warp_first = s0 + (group - (((threadIdx.x & 31)) / L));
    int beg = 0, end = 0;
    if (r < s1) {
        beg = A.ptr[r];
        end = A.ptr[r + 1];
    }
    for (int wbase = warp_first; wbase < s1; wbase += ngroups, r += ngroups) {
        // prefetch the next segment's pointers
        const int rn = r + ngroups;
        int nbeg = 0, nend = 0;
        if (rn < s1) {
            nbeg = A.ptr[rn];
            nend = A.ptr[rn + 1];
        }
        const bool active = r < s1 && (EXACT || (end - beg) <= heavy_threshold);
        typename Epi::Pre pre{};
        if (active && sub == 0) pre = epi.pre(r);
        float s = 0.f;
        if (active) s = EXACT ? seg_dot_exact(A.pairs, beg, end, vec) : seg_dot(A.pairs, beg, end, sub, L, vec);
        if (!EXACT) s = group_sum(s, L);
        if (active && sub == 0) epi.apply(r, s, pre);
        beg = nbeg;
        end = nend;
    }
}

// One segment per warp (heavy segments).
template <class Epi>
__device__ __forceinline__ void spmv_warp_seg(const SegMatrix& A, const float* __restrict__ vec, int r, Epi& epi) {
    const int lane = threadIdx.x & 31;
    typename Epi::Pre pre{};
    if (lane == 0) pre = epi.pre(r);
    float s = seg_dot(A.pairs, A.ptr[r], A.ptr[r + 1], lane, 32, vec);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
    if (lane == 0) epi.apply(r, s, pre);
}

// Grid-stride SpMV of a whole side: heavy blocks first, then light blocks.
template <bool EXACT, class Epi>
__device__ __forceinline__ void spmv_run(const SegMatrix& A, const SpmvPlan& P, const float* __restrict__ vec,
                                         Epi& epi) {
    const int wpb = blockDim.x >> 5;
    if (!EXACT && (int)blockIdx.x < P.heavy_blocks) {
        const int nw = P.heavy_blocks * wpb;
        for (int h = blockIdx.x * wpb + (threadIdx.x >> 5); h < P.heavy_count; h += nw)
            spmv_warp_seg(A, vec, P.heavy_idx[h], epi);
        return;
    }
    const int L = EXACT ? 1 : P.lanes;
    const int rank = blockIdx.x - (EXACT ? 0 : P.heavy_blocks);
    const int nblocks = gridDim.x - (EXACT ? 0 : P.heavy_blocks);
    const int gpw = 32 / L;
    const int group = (rank * wpb + (threadIdx.x >> 5)) * gpw + (threadIdx.x & 31) / L;
    spmv_groups<EXACT>(A, vec, 0, A.nseg, group, nblocks * wpb * gpw, L, P.heavy_threshold, epi);
}

// ------------------------------------------------------------------ host side
// Builds the launch plan of one side from its (host) segment pointers.
// `lanes` <= 0 picks lanes from the mean segment length.  The heavy list is
// written to `heavy` (host vector) for the caller to upload.
SpmvPlan make_plan(const std::vector<int>& ptr, int lanes, int heavy_factor, bool exact, int sm_count,
                   std::vector<int>& heavy);

// Default lanes per segment for a mean segment length.
int default_lanes(double mean_len);

}  // namespace sihg
