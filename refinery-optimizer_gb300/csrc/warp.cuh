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
// Tasks are ordered by instance and cut into GROUPS of at most kGroup tasks of
// one instance.
//
// Scheduling: every warp of the grid is a worker over the side's ACTIVE task
// list (the tasks of the instances still running, rebuilt after every
// evaluation).  Warp w starts on entry w and then takes the next entry from a
// counter of the side (one atomic per task), so the work spreads over the SMs
// as it runs instead of by a static split (see task_loop for how a launch
// tells its own counter values apart without a reset).
// Reductions stay deterministic: a task's lanes reduce their compensated
// accumulators (Acc) in a fixed butterfly into the task's slot; the warp that
// completes a group (ticket) reduces the group's task slots in task order; the
// warp that completes an instance reduces its group slots in group order,
// converts the totals to FP64 and runs the instance's controller.  No warp
// ever waits for another.
//
// Inside a task, groups of L lanes walk the segments; each lane issues kBatch
// pair loads, then kBatch gathers, then the FMAs.  The loads are software
// pipelined: the first pairs of the next segment (and the next batch inside a
// long segment) are in flight while the current batch gathers; pointers run
// two segments ahead; the epilogue operands (Epi::pre) load before the dot.
//
// Epilogue interface (Epi):
//   using Pre;  Pre pre(int seg) const          operands of a segment (global loads)
//   void begin(const Inst&)                    per-task setup (vectors to gather)
//   const float* gather(int v) const           vector gathered by the nonzero indices
//   void apply(int seg, const SegDot<NV>&, const Pre&)
//   void values(Acc (&q)[Q])                   this lane's partial reductions; resets them
//                                              (a max travels in q.s with q.c = 0)
//   void finish(State&, const double* total)   instance controller (one lane)
// The per-instance state type (Inst for the PDHG solver) has `done` and
// `refine` fields; a task of a done instance is skipped.
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

// Staged gathers.  An epilogue with `kStaged = true` and a member `staged`
// (an entry count) works in a kernel whose blocks first copied entries
// [0, staged) of the gathered vector to the start of dynamic shared memory
// (stage_prefix): gathers below `staged` read that copy.  With both sides
// renumbered by descending length the prefix holds the longest segments of
// the other side, so on skewed matrices (Zipf-like column lengths) most
// gathers of K x hit the copy instead of going to L2.
template <class Epi, class = void>
struct Staged {
    static constexpr bool value = false;
};
template <class Epi>
struct Staged<Epi, decltype(void(Epi::kStaged))> {
    static constexpr bool value = Epi::kStaged;
};

// Coherent gathers.  An epilogue with `kCoherent = true` runs inside the
// persistent step kernel, where the gathered vector was written earlier in the
// same launch (before a grid barrier): its gathers use ordinary global loads,
// which the barrier's fences order, instead of the read-only (.nc) path that
// is only valid for data no thread of the launch writes.
template <class Epi, class = void>
struct Coherent {
    static constexpr bool value = false;
};
template <class Epi>
struct Coherent<Epi, decltype(void(Epi::kCoherent))> {
    static constexpr bool value = Epi::kCoherent;
};

// Computed gathers.  An epilogue with `kPackedX = true` supplies the gathered
// value itself (`gather_x(idx)`), e.g. the primal step x'_j computed from a
// packed per-column record, instead of a load from a vector.
template <class Epi, class = void>
struct PackedX {
    static constexpr bool value = false;
};
template <class Epi>
struct PackedX<Epi, decltype(void(Epi::kPackedX))> {
    static constexpr bool value = Epi::kPackedX;
};

template <class Epi>
__device__ __forceinline__ float gather_one(const Epi& epi, const float* __restrict__ vec, int idx) {
    if constexpr (PackedX<Epi>::value) {
        return epi.gather_x(idx);
    } else if constexpr (Coherent<Epi>::value) {
        float v;
        asm volatile("ld.global.f32 %0, [%1];" : "=f"(v) : "l"(vec + idx));
        return v;
    } else if constexpr (Staged<Epi>::value) {
        // predicated loads, no branch: the shared copy below `staged`, else
        // the vector (the gathers of a batch then issue back to back)
        extern __shared__ float stage_vec[];
        const unsigned saddr = (unsigned)__cvta_generic_to_shared(stage_vec) + 4u * (unsigned)idx;
        float v;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.lt.s32 p, %1, %2;\n\t"
            "@p ld.shared.f32 %0, [%3];\n\t"
            "@!p ld.global.nc.f32 %0, [%4];\n\t}"
            : "=f"(v)
            : "r"(idx), "r"(epi.staged), "r"(saddr), "l"(vec + idx));
        return v;
    }
    return ld_vec(vec + idx);
}

// Copies v[0, n) to the start of dynamic shared memory (all threads of the
// block, then a block barrier).  n is a multiple of 4.
__device__ __forceinline__ void stage_prefix(const float* __restrict__ v, int n) {
    extern __shared__ float stage_vec[];
    if ((reinterpret_cast<uintptr_t>(v) & 15) == 0) {
        const float4* __restrict__ v4 = reinterpret_cast<const float4*>(v);
        float4* s4 = reinterpret_cast<float4*>(stage_vec);
        for (int k = threadIdx.x; k < (n >> 2); k += blockDim.x) s4[k] = __ldcg(v4 + k);
    } else {
        for (int k = threadIdx.x; k < n; k += blockDim.x) stage_vec[k] = __ldcg(v + k);
    }
    __syncthreads();
}

// Loads one batch of a lane's pairs (entries k, k + L, ..., k + (kBatch-1) L
// below `end`); the rest are zero.
__device__ __forceinline__ void load_batch(bool on, const int2* __restrict__ pairs, int k, int end, int L,
                                           int2 (&p)[kBatch]) {
#pragma unroll
    for (int u = 0; u < kBatch; ++u) p[u] = (on && k + u * L < end) ? ld_pair(pairs + k + u * L) : make_int2(0, 0);
}

// Dot products of one segment with the NV gathered vectors, this lane's share
// (entries beg+sub, +L, ...), reduced over the lane group.  `p` holds the
// lane's first batch of pairs on entry (loaded ahead by the caller); inside a
// long segment the next batch's pairs load while the current batch gathers.
// Plain: kBatch FMA chains per vector, summed pairwise (as seg_dot);
// COMP: Dot2 (two-product + two-sum) per vector.
template <int NV, bool COMP, class Epi>
__device__ __forceinline__ void seg_dots(const int2* __restrict__ pairs, int beg, int end, int sub, int L,
                                         bool active, Epi& epi, int2 (&p)[kBatch], SegDot<NV>& d) {
    float acc[NV][kBatch], s2[NV], e2[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        s2[v] = e2[v] = 0.f;
#pragma unroll
        for (int u = 0; u < kBatch; ++u) acc[v][u] = 0.f;
    }
    if (active) {
        for (int k = beg + sub;; k += kBatch * L) {
            const int kn = k + kBatch * L;
            const bool more = kn < end;
            int2 q[kBatch];
            load_batch(more, pairs, kn, end, L, q);
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                const float* __restrict__ vec = epi.gather(v);
                float g[kBatch];
#pragma unroll
                for (int u = 0; u < kBatch; ++u) g[u] = (k + u * L < end) ? gather_one(epi, vec, p[u].x) : 0.f;
#pragma unroll
                for (int u = 0; u < kBatch; ++u) {
                    if (COMP) {
                        float pr, pe, ss, se;
                        two_prod(__int_as_float(p[u].y), g[u], pr, pe);
                        two_sum(s2[v], pr, ss, se);
                        s2[v] = ss;
                        e2[v] = __fadd_rn(e2[v], __fadd_rn(pe, se));
                    } else {
                        acc[v][u] = fmaf(__int_as_float(p[u].y), g[u], acc[v][u]);
                    }
                }
            }
            if (!more) break;
#pragma unroll
            for (int u = 0; u < kBatch; ++u) p[u] = q[u];
        }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        float s = COMP ? s2[v] : (acc[v][0] + acc[v][1]) + (acc[v][2] + acc[v][3]);
        float e = e2[v];
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
// listed segments).  Software pipeline over segments: the pointers of the
// segment two ahead and the first pairs of the next segment are in flight
// while the current segment gathers.
template <int NV, bool COMP, bool LIST, class Epi>
__device__ __forceinline__ void run_task(const SegMatrix& A, const int* __restrict__ list, const Task& t,
                                         int light_max, Epi& epi) {
    static_assert(kBatch == 4, "seg_dots sums four FMA chains");
    const int L = task_lanes(t.flags);
    const int lane = threadIdx.x & 31, sub = lane & (L - 1), gpw = 32 / L;
    int k = t.seg_begin + lane / L;
    int r0 = -1, b0 = 0, e0 = 0, r1 = -1, b1 = 0, e1 = 0;
    if (k < t.seg_end) {
        r0 = LIST ? list[k] : k;
        b0 = A.ptr[r0];
        e0 = A.ptr[r0 + 1];
    }
    if (k + gpw < t.seg_end) {
        r1 = LIST ? list[k + gpw] : k + gpw;
        b1 = A.ptr[r1];
        e1 = A.ptr[r1 + 1];
    }
    bool act0 = k < t.seg_end && (LIST || e0 - b0 <= light_max);
    int2 p0[kBatch];
    load_batch(act0, A.pairs, b0 + sub, e0, L, p0);
    for (int wb = t.seg_begin; wb < t.seg_end; wb += gpw, k += gpw) {
        const int k2 = k + 2 * gpw;
        int r2 = -1, b2 = 0, e2 = 0;
        if (k2 < t.seg_end) {
            r2 = LIST ? list[k2] : k2;
            b2 = A.ptr[r2];
            e2 = A.ptr[r2 + 1];
        }
        const bool act1 = k + gpw < t.seg_end && (LIST || e1 - b1 <= light_max);
        int2 p1[kBatch];
        load_batch(act1, A.pairs, b1 + sub, e1, L, p1);
        typename Epi::Pre pre{};
        if (act0 && sub == 0) pre = epi.pre(r0);
        SegDot<NV> d;
        seg_dots<NV, COMP>(A.pairs, b0, e0, sub, L, act0, epi, p0, d);
        if (act0 && sub == 0) epi.apply(r0, d, pre);
        r0 = r1;
        b0 = b1;
        e0 = e1;
        act0 = act1;
#pragma unroll
        for (int u = 0; u < kBatch; ++u) p0[u] = p1[u];
        r1 = r2;
        b1 = b2;
        e1 = e2;
    }
}

template <int NV, bool COMP, class Epi>
__device__ __forceinline__ void run_any_task(const Side& side, const Task& t, int light_max, Epi& epi) {
    if (t.flags & kTaskList)
        run_task<NV, COMP, true>(side.A, side.list_idx, t, light_max, epi);
    else
        run_task<NV, COMP, false>(side.A, side.list_idx, t, light_max, epi);
}

// ---------------------------------------------------------------- deterministic reductions
// (s1 + c1) + (s2 + c2) with the rounding error of the leading sum kept; the
// result does not depend on the order of the operands.
__device__ __forceinline__ Acc acc_plus(const Acc& a, const Acc& b) {
    Acc r;
    float e;
    two_sum(a.s, b.s, r.s, e);
    r.c = __fadd_rn(__fadd_rn(a.c, b.c), e);
    return r;
}

__device__ __forceinline__ Acc acc_join(const Acc& a, const Acc& b, bool is_max) {
    if (is_max) {
        Acc r;
        r.s = fmaxf(a.s, b.s);
        r.c = 0.f;
        return r;
    }
    return acc_plus(a, b);
}

// Butterfly over the warp: every lane ends with the same value.
template <int Q>
__device__ __forceinline__ void warp_reduce_acc(Acc (&q)[Q], unsigned max_mask) {
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const bool is_max = (max_mask >> i) & 1u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            Acc b;
            b.s = __shfl_xor_sync(FULL_MASK, q[i].s, o);
            b.c = __shfl_xor_sync(FULL_MASK, q[i].c, o);
            q[i] = acc_join(q[i], b, is_max);
        }
    }
}

template <int Q>
__device__ __forceinline__ void store_slot(float2* slot, const Acc (&q)[Q]) {
#pragma unroll
    for (int i = 0; i < Q; ++i) slot[i] = make_float2(q[i].s, q[i].c);
}

// Ticket increment with release (the caller's earlier slot stores become
// visible before it) and acquire (the last arriver sees every other caller's
// slots): atom.acq_rel at GPU scope, no separate fence.
__device__ __forceinline__ unsigned ticket_add(unsigned* t) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(t) : "memory");
    return old;
}

template <int Q>
__device__ __forceinline__ void load_slot_join(const float2* slot, Acc (&q)[Q], unsigned max_mask) {
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        const float2 v = __ldcg(slot + i);
        Acc b;
        b.s = v.x;
        b.c = v.y;
        q[i] = acc_join(q[i], b, (max_mask >> i) & 1u);
    }
}

// After a task of instance t.inst has left its lane partials in q (all lanes):
// writes the task slot and runs the group / instance completion.  Returns
// true (in every lane) on the warp that completed the instance; `total` then
// holds the instance's FP64 totals.
template <int Q>
__device__ bool task_complete(const Side& side, int ti, int inst, Acc (&q)[Q], unsigned max_mask,
                              double (&total)[Q]) {
    const int lane = threadIdx.x & 31;
    warp_reduce_acc<Q>(q, max_mask);
    const int g = side.task_group[ti];
    const int gb = side.group_begin[g], ge = side.group_begin[g + 1];
    unsigned last = 0;
    if (lane == 0) {
        store_slot<Q>(side.task_part + (size_t)ti * kQ, q);
        last = ticket_add(&side.group_tickets[g]) + 1u == (unsigned)(ge - gb);
    }
    last = __shfl_sync(FULL_MASK, last, 0);
    __syncwarp();  // orders lane 0's acquire before the other lanes' slot loads
    if (!last) return false;
    // this warp completed group g: reduce its task slots in task order
    Acc v[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) v[i].reset();
    if (gb + lane < ge) load_slot_join<Q>(side.task_part + (size_t)(gb + lane) * kQ, v, max_mask);
    warp_reduce_acc<Q>(v, max_mask);
    unsigned ilast = 0;
    if (lane == 0) {
        side.group_tickets[g] = 0u;
        store_slot<Q>(side.group_part + (size_t)g * kQ, v);
        const int ngr = side.inst_group_begin[inst + 1] - side.inst_group_begin[inst];
        ilast = ticket_add(&side.tickets[inst]) + 1u == (unsigned)ngr;
    }
    ilast = __shfl_sync(FULL_MASK, ilast, 0);
    __syncwarp();
    if (!ilast) return false;
    // this warp completed the instance: reduce its group slots (lane k takes
    // groups k, k + 32, ... in order, then the butterfly)
    const int ib = side.inst_group_begin[inst], ie = side.inst_group_begin[inst + 1];
#pragma unroll
    for (int i = 0; i < Q; ++i) v[i].reset();
    // U slots per lane in flight at once (the loop is latency-bound: one
    // instance can have ~1000 groups); the join order stays k, k + 32, ...
    constexpr int U = Q <= 2 ? 8 : (Q <= 4 ? 4 : 2);
    for (int k0 = ib + lane; k0 < ie; k0 += 32 * U) {
        float2 buf[U][Q];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + 32 * u;
#pragma unroll
            for (int i = 0; i < Q; ++i)
                buf[u][i] = k < ie ? __ldcg(side.group_part + (size_t)k * kQ + i) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (k0 + 32 * u >= ie) break;
#pragma unroll
            for (int i = 0; i < Q; ++i) {
                Acc b;
                b.s = buf[u][i].x;
                b.c = buf[u][i].y;
                v[i] = acc_join(v[i], b, (max_mask >> i) & 1u);
            }
        }
    }
    warp_reduce_acc<Q>(v, max_mask);
#pragma unroll
    for (int i = 0; i < Q; ++i) total[i] = (double)v[i].s + (double)v[i].c;
    if (lane == 0) side.tickets[inst] = 0u;
    return true;
}

// Worker loop of one warp over the side's tasks.  `body(t, S)` does the work
// of one task (all lanes), leaving partials in `epi`.
template <int Q, class Epi, class State, class Body>
__device__ __forceinline__ void task_loop(const Side& side, State* st, Epi& epi, unsigned max_mask, Body&& body) {
    const int lane = threadIdx.x & 31;
    const int nw = gridDim.x * (blockDim.x >> 5);
    const int nact = *side.nactive;  // tasks of the running instances
    int pos = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    while (pos < nact) {
        // the next position is fetched while this task runs.  Every launch
        // takes exactly nact values from the counter (nact - nw positions
        // beyond the static first ones, then one past-the-end value per warp
        // that entered), and launches on a side never overlap, so the value
        // modulo nact is this launch's own sequence number; the compaction
        // after each evaluation zeroes the counter.
        int next = 0;
        if (lane == 0) next = (int)(atomicAdd(&side.counters[0], 1u) % (unsigned)nact) + nw;
        const int ti = nact == side.ntasks ? pos : side.active[pos];
        const Task t = side.tasks[ti];
        State& S = st[t.inst];
        if (!S.done) {  // uniform over the warp; it only changes after the instance's last task
            body(t, S);
            if constexpr (Q > 0) {  // Q = 0: no reductions, no tickets
                Acc q[Q];
                epi.values(q);
                double tot[Q];
                if (task_complete<Q>(side, ti, t.inst, q, max_mask, tot) && lane == 0) epi.finish(S, tot);
                __syncwarp();
            }
        }
        pos = __shfl_sync(FULL_MASK, next, 0);
    }
}

template <int Q, class Epi, class State, class Prep, class Body>
__device__ __forceinline__ void task_loop(const Side& side, State* st, Epi& epi, unsigned max_mask, Prep&&,
                                          Body&& body) {
    task_loop<Q>(side, st, epi, max_mask, body);
}

// SpMV engine: the tasks of the side with the epilogue Epi.  With ALLOW_COMP
// the tasks of an instance with `refine` set run compensated (Dot2).
template <int NV, bool ALLOW_COMP, int Q, class Epi, class State>
__device__ __forceinline__ void spmv_engine(const Side& side, State* st, Epi& epi, unsigned max_mask) {
    task_loop<Q>(side, st, epi, max_mask, [&](const Task& t, const State& S) {
        epi.begin(S);
        const int lmax = side.light_max[t.inst];
        if (ALLOW_COMP && S.refine)
            run_any_task<NV, true>(side, t, lmax, epi);
        else
            run_any_task<NV, false>(side, t, lmax, epi);
    });
}

// Elementwise pass over every column (is_col) and row of the running
// instances: blocks take chunks of kChunk consecutive elements of one
// instance, threads stride through a chunk (coalesced).  `prep(S)` turns the
// instance state into the chunk's scalars once per block, on one thread
// (FP64 arithmetic and conversions stay out of the element loop);
// `f(is_col, scalars, k)` does one element.
template <class State, class Prep, class F>
__device__ __forceinline__ void for_each_element(const Chunks& ch, State* st, Prep&& prep, F&& f) {
    using Scalars = decltype(prep(st[0]));
    __shared__ Scalars sh;  // prep runs on one thread (FP64 is slow on this part)
    const int nact = *ch.nactive;
    for (int c = blockIdx.x; c < nact; c += gridDim.x) {
        const int4 d = ch.chunks[ch.active[c]];  // begin, end, instance, is_col
        const State& S = st[d.z];
        if (S.done) continue;  // uniform over the block
        const bool is_col = d.w != 0;
        __syncthreads();
        if (threadIdx.x == 0) sh = prep(S);
        __syncthreads();
        const Scalars sc = sh;
        for (int r = d.x + threadIdx.x; r < d.y; r += blockDim.x) f(is_col, sc, r);
    }
}

}  // namespace sihg
