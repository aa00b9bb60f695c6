// Task engine of the mixed-precision / batched path.
//
// Work units on one side (rows of A for K x, columns for K^T y):
//   * a LIGHT task is a contiguous range of segments of one instance with at
//     most task_nnz nonzeros; segments longer than the instance's light_max
//     are skipped in it;
//   * a LIST task lists (list_idx[seg_begin..seg_end)) longer segments of one
//     instance and one length class, so that the lane groups of a warp get
//     segments within a factor 2 of each other (Zipf-like columns stay
//     balanced); its lane-group width grows with the class.
// Tasks are ordered by instance.  Each block owns a contiguous, nonzero-balanced
// range of tasks, cut into RUNS (the block's tasks of one instance).  The
// warps of the block share a run's tasks; every lane keeps FP32 compensated
// accumulators (Acc).  After a run the block reduces them once (FP64 only at
// this step) into the run's slot and takes a ticket of the instance; the block
// completing the instance reduces the instance's run slots in order
// (deterministic) and runs its controller.
//
// Inside a task, groups of L lanes walk the segments; each lane issues kBatch
// pair loads, then kBatch gathers, then the FMAs; the next segment's pointers
// and the epilogue operands (Epi::pre) are loaded before the current dot.
//
// Epilogue interface (Epi):
//   using Pre;  Pre pre(int seg) const          operands of a segment (global loads)
//   void begin(const Inst&)                    per-run setup (vectors to gather)
//   const float* gather(int v) const           vector gathered by the nonzero indices
//   void apply(int seg, const SegDot<NV>&, const Pre&)
//   template <int Q> values(double (&q)[Q])    this thread's partial reductions; reset them
//   void finish(Inst&, const double* total)    instance controller (one thread)
#pragma once

#include "mixed.h"
#include "spmv.cuh"

namespace sihg {

template <int NV>
struct SegDot {
    float s[NV];
    float e[NV];
    // hi + lo rounded to float
    __device__ __forceinline__ float f(int v) const { return __fadd_rn(s[v], e[v]); }
};

template <int NV, bool COMP, class Epi>
__device__ __forceinline__ void seg_group_dot(const SegMatrix& A, int beg, int end, int sub, int L, bool active,
                                              Epi& epi, SegDot<NV>& d) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        float s = 0.f, e = 0.f;
        if (active) {
            if (COMP)
                seg_dot2(A.pairs, beg, end, sub, L, epi.gather(v), s, e);
            else
                s = seg_dot(A.pairs, beg, end, sub, L, epi.gather(v));
        }
        if (COMP)
            group_sum2(s, e, L);
        else
            s = group_sum(s, L);
        d.s[v] = s;
        d.e[v] = e;
    }
}

// One task on one warp: groups of L lanes walk its segments (a light task's
// contiguous range, skipping segments longer than light_max, or a list task's
// listed segments).
template <int NV, bool COMP, bool LIST, class Epi>
__device__ __forceinline__ void run_task(const SegMatrix& A, const int* __restrict__ list, const Task& t,
                                         int light_max, Epi& epi) {
    const int L = task_lanes(t.flags);
    const int lane = threadIdx.x & 31, sub = lane & (L - 1), gpw = 32 / L;
    int k = t.seg_begin + lane / L;
    int r = -1, beg = 0, end = 0;
    if (k < t.seg_end) {
        r = LIST ? list[k] : k;
        beg = A.ptr[r];
        end = A.ptr[r + 1];
    }
    for (int wb = t.seg_begin; wb < t.seg_end; wb += gpw, k += gpw) {
        const int kn = k + gpw;
        int rn = -1, nbeg = 0, nend = 0;
        if (kn < t.seg_end) {  // next segment's pointers in flight during this one
            rn = LIST ? list[kn] : kn;
            nbeg = A.ptr[rn];
            nend = A.ptr[rn + 1];
        }
        const bool active = k < t.seg_end && (LIST || end - beg <= light_max);
        typename Epi::Pre pre{};
        if (active && sub == 0) pre = epi.pre(r);
        SegDot<NV> d;
        seg_group_dot<NV, COMP>(A, beg, end, sub, L, active, epi, d);
        if (active && sub == 0) epi.apply(r, d, pre);
        r = rn;
        beg = nbeg;
        end = nend;
    }
}

template <int NV, bool COMP, class Epi>
__device__ __forceinline__ void run_any_task(const Side& side, const Task& t, int light_max, Epi& epi) {
    if (t.flags & kTaskList)
        run_task<NV, COMP, true>(side.A, side.list_idx, t, light_max, epi);
    else
        run_task<NV, COMP, false>(side.A, side.list_idx, t, light_max, epi);
}

// Reduction of one run (all threads of the block): block-reduces Q values
// (sum, or max for the bits of max_mask) into the run's slot and takes a ticket
// of the instance.  Returns true (in every thread) on the block that completed
// the instance; `total` (thread 0) then holds the instance totals, reduced
// over its run slots in order.
template <int Q>
__device__ bool run_reduce(const Side& side, int run, int inst, const double (&q)[Q], unsigned max_mask,
                           double (&total)[Q]) {
    __shared__ double red[Q][32];
    __shared__ bool s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const bool is_max = (max_mask >> i) & 1u;
        const double v = is_max ? warp_maxd(q[i]) : warp_sum(q[i]);
        if (lane == 0) red[i][warp] = v;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const bool is_max = (max_mask >> i) & 1u;
            double v = lane < nwarps ? red[i][lane] : 0.0;
            v = is_max ? warp_maxd(v) : warp_sum(v);
            if (lane == 0) side.partials[(size_t)run * kQ + i] = v;
        }
        if (lane == 0) {
            __threadfence();
            const unsigned ib = side.inst_run_begin[inst], ie = side.inst_run_begin[inst + 1];
            const unsigned old = atomicAdd(&side.tickets[inst], 1u);
            s_last = old + 1u == ie - ib;
        }
    }
    __syncthreads();
    const bool last = s_last;
    if (last) {
        __threadfence();
        const int ib = side.inst_run_begin[inst], ie = side.inst_run_begin[inst + 1];
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const bool is_max = (max_mask >> i) & 1u;
            double acc = 0.0;
            for (int k = ib + (int)threadIdx.x; k < ie; k += blockDim.x) {
                const double v = __ldcg(&side.partials[(size_t)k * kQ + i]);
                acc = is_max ? fmax(acc, v) : acc + v;
            }
            acc = is_max ? warp_maxd(acc) : warp_sum(acc);
            if (lane == 0) red[i][warp] = acc;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                const bool is_max = (max_mask >> i) & 1u;
                double acc = 0.0;
                for (int w = 0; w < nwarps; ++w) acc = is_max ? fmax(acc, red[i][w]) : acc + red[i][w];
                total[i] = acc;
            }
            side.tickets[inst] = 0u;
        }
    }
    __syncthreads();
    return last;
}

// Runs the block's runs.  With ALLOW_COMP the tasks of an instance with
// `refine` set run compensated (Dot2).  Q = reduced values, max_mask marks the
// ones reduced by max instead of sum.
template <int NV, bool ALLOW_COMP, int Q, class Epi>
__device__ void block_engine(const Side& side, Inst* st, Epi& epi, unsigned max_mask) {
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int rb = side.block_run_begin[blockIdx.x], re = side.block_run_begin[blockIdx.x + 1];
    for (int run = rb; run < re; ++run) {
        const Run R = side.runs[run];
        Inst& S = st[R.inst];
        if (S.done) continue;  // uniform: the flag only changes after the instance's last run
        epi.begin(S);
        const bool comp = ALLOW_COMP && S.refine;
        const int lmax = side.light_max[R.inst];
        for (int ti = R.task_begin + warp; ti < R.task_end; ti += nwarps) {
            const Task t = side.tasks[ti];
            if (comp)
                run_any_task<NV, true>(side, t, lmax, epi);
            else
                run_any_task<NV, false>(side, t, lmax, epi);
        }
        double q[Q], tot[Q];
        epi.values(q);
        if (run_reduce<Q>(side, run, R.inst, q, max_mask, tot) && threadIdx.x == 0) epi.finish(S, tot);
        __syncthreads();
    }
}

// Elementwise pass: warp-strided over the light tasks of both sides (columns
// first; light tasks cover every segment), lane-strided over their segments.
template <class F>
__device__ __forceinline__ void for_each_segment_both(const Side& cols, const Side& rows, Inst* st, F&& f) {
    const int wpb = blockDim.x >> 5;
    const int gw = blockIdx.x * wpb + (threadIdx.x >> 5), nw = gridDim.x * wpb;
    const int lane = threadIdx.x & 31;
    for (int ti = gw; ti < cols.ntasks + rows.ntasks; ti += nw) {
        const bool is_col = ti < cols.ntasks;
        const Side& sd = is_col ? cols : rows;
        const Task t = sd.tasks[is_col ? ti : ti - cols.ntasks];
        if (t.flags & kTaskList) continue;
        const Inst& S = st[t.inst];
        if (S.done) continue;
        for (int r = t.seg_begin + lane; r < t.seg_end; r += 32) f(is_col, S, r);
    }
}

}  // namespace sihg
