// Sparse matrix-vector core of the PDHG engine.
//
// A "segment matrix" is one side of the LP matrix: the rows of A (CSR, used
// for A x) or the columns of A (CSC, used for A^T y).  Entries are stored as
// packed 8-byte pairs {index, float bits} so that one 64-bit load brings both
// the index and the value of a nonzero (one load instruction and one 32-byte
// sector per 4 nonzeros of a segment).
//
// Work split (one launch):
//   * light segments (length <= heavy_threshold) are handled by groups of
//     `lanes` consecutive threads (1..32), in natural segment order, so the
//     per-segment epilogue reads and writes its vectors coalesced;
//   * heavy segments (longer) are listed in heavy_idx and handled by whole
//     warps in the first `heavy_blocks` blocks of the grid.
// The epilogue functor `epi(seg, dot)` runs once per segment on the lane that
// owns the reduced dot product; it fuses the PDHG update of that row/column.
//
// EXACT mode reproduces the reference kernels' arithmetic
// (core/src/gpu/cuda_pdhg.cu:14-49): one thread per segment, products and
// sums in entry order, no fused multiply-add.
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

__device__ __forceinline__ int2 ld_pair(const int2* p) {
    int2 v;
    asm("ld.global.nc.L1::no_allocate.v2.s32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ float ld_vec(const float* p) { return __ldg(p); }

// Dot product of one segment with `vec`, this lane's share: entries
// beg + lane0, beg + lane0 + L, ...  (four independent loads in flight).
__device__ __forceinline__ float seg_dot(const int2* __restrict__ pairs, int beg, int end, int lane0, int L,
                                         const float* __restrict__ vec) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int k = beg + lane0;
    for (; k + 3 * L < end; k += 4 * L) {
        const int2 p0 = ld_pair(pairs + k), p1 = ld_pair(pairs + k + L);
        const int2 p2 = ld_pair(pairs + k + 2 * L), p3 = ld_pair(pairs + k + 3 * L);
        s0 = fmaf(__int_as_float(p0.y), ld_vec(vec + p0.x), s0);
        s1 = fmaf(__int_as_float(p1.y), ld_vec(vec + p1.x), s1);
        s2 = fmaf(__int_as_float(p2.y), ld_vec(vec + p2.x), s2);
        s3 = fmaf(__int_as_float(p3.y), ld_vec(vec + p3.x), s3);
    }
    for (; k < end; k += L) {
        const int2 p0 = ld_pair(pairs + k);
        s0 = fmaf(__int_as_float(p0.y), ld_vec(vec + p0.x), s0);
    }
    return (s0 + s1) + (s2 + s3);
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

template <bool EXACT, class Epi>
__device__ __forceinline__ void spmv_light(const SegMatrix& A, const SpmvPlan& P, const float* __restrict__ vec,
                                           int rank, int nblocks, Epi& epi) {
    const int L = EXACT ? 1 : P.lanes;
    const int lane = threadIdx.x & 31;
    const int sub = lane & (L - 1);
    const int gpw = 32 / L;
    const int wpb = blockDim.x >> 5;
    const int wid = rank * wpb + (threadIdx.x >> 5);
    const int nw = nblocks * wpb;
    for (int base = wid * gpw; base < A.nseg; base += nw * gpw) {
        const int r = base + lane / L;
        float s = 0.f;
        bool active = false;
        if (r < A.nseg) {
            const int beg = A.ptr[r], end = A.ptr[r + 1];
            active = EXACT || (end - beg) <= P.heavy_threshold;
            if (active) s = EXACT ? seg_dot_exact(A.pairs, beg, end, vec) : seg_dot(A.pairs, beg, end, sub, L, vec);
        }
        if (!EXACT) {
            for (int o = L >> 1; o > 0; o >>= 1) s += __shfl_down_sync(FULL_MASK, s, o, L);
        }
        if (active && sub == 0) epi(r, s);
    }
}

template <class Epi>
__device__ __forceinline__ void spmv_heavy(const SegMatrix& A, const SpmvPlan& P, const float* __restrict__ vec,
                                           int rank, int nblocks, Epi& epi) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const int wid = rank * wpb + (threadIdx.x >> 5);
    const int nw = nblocks * wpb;
    for (int h = wid; h < P.heavy_count; h += nw) {
        const int r = P.heavy_idx[h];
        float s = seg_dot(A.pairs, A.ptr[r], A.ptr[r + 1], lane, 32, vec);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
        if (lane == 0) epi(r, s);
    }
}

// Runs the whole SpMV of one launch: heavy blocks first, then light blocks.
template <bool EXACT, class Epi>
__device__ __forceinline__ void spmv_run(const SegMatrix& A, const SpmvPlan& P, const float* __restrict__ vec,
                                         Epi& epi) {
    if (!EXACT && (int)blockIdx.x < P.heavy_blocks)
        spmv_heavy(A, P, vec, blockIdx.x, P.heavy_blocks, epi);
    else
        spmv_light<EXACT>(A, P, vec, blockIdx.x - (EXACT ? 0 : P.heavy_blocks),
                          gridDim.x - (EXACT ? 0 : P.heavy_blocks), epi);
}

// ------------------------------------------------------------------ host side
// Builds the launch plan of one side from its (host) segment pointers.
// `lanes` <= 0 picks lanes from the mean segment length.  The heavy list is
// written to `heavy` (host vector) for the caller to upload.
SpmvPlan make_plan(const std::vector<int>& ptr, int lanes, int heavy_factor, bool exact, int sm_count,
                   std::vector<int>& heavy);

}  // namespace sihg
