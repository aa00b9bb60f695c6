// Mixed-precision restarted adaptive PDHG on the device, for one LP or a batch
// of independent LPs (block-diagonal concatenation, per-instance state).
//
// Algorithm (the reference specifies it in docs/gpu_pdhg.md:29-57; the code
// path it ships does not have it, so the adaptive pieces follow the published
// PDLP method: Applegate et al., "Practical large-scale linear programming
// using primal-dual hybrid gradient", NeurIPS 2021, and its GPU form cuPDLP,
// Lu & Yang 2023):
//   scaling   Ruiz equilibration (inf-norm, `ruiz_iterations` passes) then one
//             Pock-Chambolle pass (alpha = 1) on the device;
//   step      tau = eta / omega, sigma = eta * omega; eta adapted every step:
//             eta_bar = (omega |dx|^2 + |dy|^2 / omega) / (2 |dx' K' dy|),
//             accept when eta <= eta_bar, next
//             eta = min((1 - (k+1)^-0.3) eta_bar, (1 + (k+1)^-0.6) eta);
//   restart   every `eval_frequency` steps: KKT of the current and of the
//             step-weighted average iterate; restart to the better one on
//             sufficient (0.2), necessary-without-progress (0.8) or artificial
//             (0.36 of all steps) decay of the weighted KKT error;
//   weight    at a restart omega <- exp(th log(|dy|/|dx|) + (1 - th) log omega)
//             from the distances moved since the previous restart, th =
//             `primal_weight_smoothing` (PDLP's 0.5 by default);
//   stop      relative KKT of docs/gpu_pdhg.md:51-57 (inf-norms, original
//             space) of the current or average point <= tolerances.
// Precision: matrix, iterates and SpMV products in FP32; every reduction
// (norms, objectives, gap, step-size terms, primal weight) in FP64; the
// evaluation SpMVs use compensated Dot2 sums near the tolerance.
//
// PDHG sign: y is the reference's y_pdhg (= -simplex dual), the dual step is
// the reference's y <- sigma (w - clip(w, rl, ru)), w = K xbar + y / sigma
// (core/src/gpu/cuda_pdhg.cu:82-103), with K xbar = 2 K x' - K x by linearity.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>

#include "mixed.h"
#include "gridsync.cuh"
#include "warp.cuh"

namespace sihg {

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ float* pick(float* a, float* b, int sel) { return sel ? b : a; }
__device__ __forceinline__ bool fin(float v) { return !isinf(v); }

// Programmatic dependent launch.  The step kernels are launched with
// programmatic stream serialization (launch_chained): their blocks may be
// scheduled while the previous kernel in the stream finishes, and wait here,
// before their first memory access, until it has completed and its writes are
// visible; then they let the next kernel be scheduled.  Without the launch
// attribute both instructions do nothing.
__device__ __forceinline__ void chain_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// a - (s + e) for a float a and a float-float s + e, without losing the low part
__device__ __forceinline__ float diff_ff(float a, float s, float e) {
    float h, l;
    two_sum(a, -s, h, l);
    return __fadd_rn(h, __fsub_rn(l, e));
}

// Bound violation of the float-float row activity s + e (0 inside [rl, ru]).
__device__ __forceinline__ float row_violation(float s, float e, float rl, float ru) {
    float v = 0.f;
    if (fin(rl)) v = fmaxf(v, diff_ff(rl, s, e));
    if (fin(ru)) v = fmaxf(v, -diff_ff(ru, s, e));
    return v;
}

// dual objective contribution of a row (scaling invariant), PDHG sign y
__device__ __forceinline__ void row_dual_term(Acc& acc, float y, float rl, float ru) {
    if (y < 0.f && fin(rl)) acc.add_prod(-y, rl);
    if (y > 0.f && fin(ru)) acc.add_prod(-y, ru);
}

// ---------------------------------------------------------------- step kernels
// Elementwise part of a step.  Columns: pending float-float average update of
// x, then x' = clip(x - tau (c + K^T y), l, u).  Rows: pending average update of y.
// Scalars of an instance for the elementwise passes (computed once per chunk).
struct StepScalars {
    int cur, avg, flag;
    float w, tau;
};

__device__ __forceinline__ StepScalars step_scalars(const Inst& S) {
    return StepScalars{S.cur, S.avg_pending, S.restart_flag, (float)S.avg_w, (float)(S.eta / S.omega)};
}

template <int U>
__device__ __forceinline__ void step_primal_body(const Chunks& ch, const Vecs& V, const Inst* st) {
    // chunks as for_each_element; every thread loads the operands of U
    // elements of its chunk before it stores any of them (the stores would
    // otherwise keep the next element's loads behind them: one DRAM latency
    // per element)
    __shared__ StepScalars sh;
    const int nact = *ch.nactive;
    for (int c = blockIdx.x; c < nact; c += gridDim.x) {
        const int4 d = ch.chunks[ch.active[c]];  // begin, end, instance, is_col
        const Inst& I = st[d.z];
        if (I.done) continue;  // uniform over the block
        // one thread turns the FP64 state into the chunk's scalars (an FP64
        // division: per thread it would keep the slow FP64 pipe busy)
        __syncthreads();
        if (threadIdx.x == 0) sh = step_scalars(I);
        __syncthreads();
        const StepScalars S = sh;
        if (d.w) {
            const float* xs = pick(V.x0, V.x1, S.cur);
            const float* kt = pick(V.kty0, V.kty1, S.cur);
            float* xn = pick(V.x0, V.x1, S.cur ^ 1);
            for (int r0 = d.x + threadIdx.x; r0 < d.y; r0 += U * blockDim.x) {
                float xv[U], cv[U], kv[U], lv[U], uv[U];
                float2 av[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int r = r0 + u * blockDim.x;
                    if (r < d.y) {
                        xv[u] = xs[r];
                        cv[u] = V.c[r];
                        kv[u] = kt[r];
                        lv[u] = V.l[r];
                        uv[u] = V.u[r];
                        if (S.avg) av[u] = V.x_acc[r];
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int r = r0 + u * blockDim.x;
                    if (r < d.y) {
                        if (S.avg) V.x_acc[r] = ff_axpy(av[u], S.w, xv[u]);
                        const float v = fmaf(-S.tau, cv[u] + kv[u], xv[u]);
                        xn[r] = fminf(fmaxf(v, lv[u]), uv[u]);
                    }
                }
            }
        } else if (S.avg) {
            const float* ys = pick(V.y0, V.y1, S.cur);
            for (int r0 = d.x + threadIdx.x; r0 < d.y; r0 += U * blockDim.x) {
                float yv[U];
                float2 av[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int r = r0 + u * blockDim.x;
                    if (r < d.y) {
                        yv[u] = ys[r];
                        av[u] = V.y_acc[r];
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int r = r0 + u * blockDim.x;
                    if (r < d.y) V.y_acc[r] = ff_axpy(av[u], S.w, yv[u]);
                }
            }
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_step_primal(int B, Chunks ch, Vecs V, Inst* __restrict__ st) {
    chain_wait();
    step_primal_body<4>(ch, V, st);
}

// The step-size schedule factors k^-0.6 and k^-0.3 of attempt k (k =
// attempts + 2).  FP64 pow is slow on this part (a chain of FP64 operations on
// a pipe that issues two per SM per clock), so the set-up tabulates both for
// every k the iteration limit reaches (up to kPowTable entries; beyond, pow
// runs on the device as before); the table holds the same pow results.
constexpr int kPowTable = 1 << 20;

__global__ void k_pow_table(int n, double2* __restrict__ tab) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        tab[k] = make_double2(pow((double)k, -0.6), pow((double)k, -0.3));
}

__device__ __forceinline__ void schedule_pows(Inst& S, const Vecs& V) {
    const long long k = S.attempts + 2;
    if (k < V.pow_n) {
        const double2 p = V.pow_tab[k];
        S.pow06 = p.x;
        S.pow03 = p.y;
    } else {
        S.pow06 = pow((double)k, -0.6);
        S.pow03 = pow((double)k, -0.3);
    }
}

// Thread 0 of block b loads the factors of instances b, b + grid, ... at the
// start of the A x kernel for the controller at the end of the A^T y kernel.
__device__ __forceinline__ void step_schedule_pows(int B, Inst* __restrict__ st, const Vecs& V) {
    if (threadIdx.x != 0) return;
    for (int b = blockIdx.x; b < B; b += gridDim.x) {
        Inst& S = st[b];
        if (S.done) continue;
        schedule_pows(S, V);
    }
}

// Row epilogue of a step: K x' arrives as the dot product; dual update with
// K xbar = 2 K x' - K x (cuda_pdhg.cu:82-103 form, PDHG sign).
struct DualStepEpi {
    Vecs V;
    const float *xg, *kx, *y;
    float *kxn, *yn;
    float sigma;
    Acc dy2;
    struct Pre { float kx, y, rl, ru; };
    __device__ Pre pre(int i) const { return Pre{kx[i], y[i], V.rl[i], V.ru[i]}; }
    __device__ void begin(const Inst& S) {
        xg = pick(V.x0, V.x1, S.cur ^ 1);
        kx = pick(V.kx0, V.kx1, S.cur);
        y = pick(V.y0, V.y1, S.cur);
        kxn = pick(V.kx0, V.kx1, S.cur ^ 1);
        yn = pick(V.y0, V.y1, S.cur ^ 1);
        sigma = (float)(S.eta * S.omega);
    }
    __device__ const float* gather(int) const { return xg; }
    __device__ void apply(int i, const SegDot<1>& d, const Pre& p) {
        const float kxp = d.f(0);  // hi + lo when compensated
        const float wv = (2.0f * kxp - p.kx) + p.y / sigma;
        const float yv = sigma * (wv - fminf(fmaxf(wv, p.rl), p.ru));
        kxn[i] = kxp;
        yn[i] = yv;
        const float dy = yv - p.y;
        dy2.add(dy * dy);
    }
    __device__ void values(Acc (&q)[1]) {
        q[0] = dy2;
        dy2.reset();
    }
    __device__ void finish(Inst& S, const double* tot) { S.dy2 = tot[0]; }
};

__global__ void __launch_bounds__(kThreads, 4) k_step_dual(int B, Side rows, Vecs V, Inst* __restrict__ st) {
    chain_wait();
    step_schedule_pows(B, st, V);
    DualStepEpi epi{V};
    spmv_engine<1, true, 1>(rows, st, epi, 0u);
}

// Step-size controller of one instance (PDLP adaptive step), one thread.
__device__ void step_controller(Inst& S, double dx2, double inter) {
    const double om = S.omega;
    const double movement = om * dx2 + S.dy2 / om;
    const double ai = fabs(inter);
    const double eta_bar = ai > 0.0 ? movement / (2.0 * ai) : INFINITY;
    // PDLP counts iterations from 1: the base k = attempts + 2 is at least 2;
    // k^-0.6 and k^-0.3 were computed by the A x kernel of this step
    const double eta = S.eta;
    const double grow = (1.0 + S.pow06) * eta;
    const double eta_next = isinf(eta_bar) ? grow : fmin((1.0 - S.pow03) * eta_bar, grow);
    S.attempts += 1;
    if (!(movement == movement) || !(inter == inter)) {  // NaN: stop as a numerical failure
        S.done = 3;
        return;
    }
    if (eta <= eta_bar) {
        S.cur ^= 1;
        S.steps += 1;
        S.since_restart += 1;
        S.W += eta;
        S.avg_w = eta / S.W;
        S.avg_pending = 1;
    } else {
        S.rejections += 1;
        S.avg_pending = 0;
    }
    S.eta = eta_next;
}

// Column epilogue of a step: K^T y' as the dot product; interaction and
// movement terms of the adaptive step.  The warp completing an instance runs
// its step-size controller.
struct KtyStepEpi {
    Vecs V;
    const float *yg, *x, *xn, *kty;
    float* ktyn;
    Acc inter, dx2;
    struct Pre { float x, xn, kty; };
    __device__ Pre pre(int j) const { return Pre{x[j], xn[j], kty[j]}; }
    __device__ void begin(const Inst& S) {
        yg = pick(V.y0, V.y1, S.cur ^ 1);
        x = pick(V.x0, V.x1, S.cur);
        xn = pick(V.x0, V.x1, S.cur ^ 1);
        kty = pick(V.kty0, V.kty1, S.cur);
        ktyn = pick(V.kty0, V.kty1, S.cur ^ 1);
    }
    __device__ const float* gather(int) const { return yg; }
    __device__ void apply(int j, const SegDot<1>& d, const Pre& p) {
        const float k = d.f(0);
        ktyn[j] = k;
        const float dx = p.xn - p.x;
        inter.add(dx * (k - p.kty));
        dx2.add(dx * dx);
    }
    __device__ void values(Acc (&q)[2]) {
        q[0] = inter;
        q[1] = dx2;
        inter.reset();
        dx2.reset();
    }
    __device__ void finish(Inst& S, const double* tot) { step_controller(S, tot[1], tot[0]); }
};

__global__ void __launch_bounds__(kThreads, 4) k_step_kty(Side cols, Vecs V, Inst* __restrict__ st) {
    chain_wait();
    KtyStepEpi epi{V};
    spmv_engine<1, true, 2>(cols, st, epi, 0u);
}

// Staged variants of the two step SpMVs (single LP): one block of
// kStagedThreads per SM copies the first `staged` entries (a multiple of 4)
// of the gathered vector to shared memory, then runs the same tasks with
// gathers below `staged` served from the copy.  Instance 0's `cur` does not
// change before the last task of the launch (the controller flips it after).
struct DualStepEpiStaged : DualStepEpi {
    static constexpr bool kStaged = true;
    int staged;
};
struct KtyStepEpiStaged : KtyStepEpi {
    static constexpr bool kStaged = true;
    int staged;
};

__global__ void __launch_bounds__(kStagedThreads, 1)
    k_step_dual_staged(int B, Side rows, Vecs V, Inst* __restrict__ st, int staged) {
    chain_wait();
    stage_prefix(pick(V.x0, V.x1, st[0].cur ^ 1), staged);
    step_schedule_pows(B, st, V);
    DualStepEpiStaged epi{{V}, staged};
    spmv_engine<1, true, 1>(rows, st, epi, 0u);
}

__global__ void __launch_bounds__(kStagedThreads, 1)
    k_step_kty_staged(Side cols, Vecs V, Inst* __restrict__ st, int staged) {
    chain_wait();
    stage_prefix(pick(V.y0, V.y1, st[0].cur ^ 1), staged);
    KtyStepEpiStaged epi{{V}, staged};
    spmv_engine<1, true, 2>(cols, st, epi, 0u);
}

// Persistent form of the step loop (options.persistent): one cooperative
// launch runs `nsteps` steps, each as the three phases of the kernels above
// (elementwise primal step, K x' with the dual step, K^T y' with the step-size
// controller) separated by grid barriers instead of kernel boundaries.  The
// gathered vectors are written inside the launch, so the epilogues gather
// through the coherent path.  Same tasks, same reduction order and same
// controller as the separate kernels, so the iterates are bit-identical.
struct DualStepEpiCoherent : DualStepEpi {
    static constexpr bool kCoherent = true;
};
struct KtyStepEpiCoherent : KtyStepEpi {
    static constexpr bool kCoherent = true;
};

__global__ void __launch_bounds__(kThreads, 4)
    k_steps_persistent(int B, int nsteps, Chunks ch, Side rows, Side cols, Vecs V, Inst* st, GridBar gb) {
    if (ld_status(gb.status) != 0) return;  // an earlier launch of this run timed out
    unsigned long long gen = grid_start(gb);
    for (int k = 0; k < nsteps; ++k) {
        step_primal_body<2>(ch, V, st);
        if (!grid_barrier(gb, gen)) return;
        step_schedule_pows(B, st, V);
        {
            DualStepEpiCoherent epi{{V}};
            spmv_engine<1, true, 1>(rows, st, epi, 0u);
        }
        if (!grid_barrier(gb, gen)) return;
        {
            KtyStepEpiCoherent epi{{V}};
            spmv_engine<1, true, 2>(cols, st, epi, 0u);
        }
        if (k + 1 < nsteps && !grid_barrier(gb, gen)) return;
    }
}

// ---------------------------------------------------------------- single-LP persistent form
// For one LP whose steps are latency-bound (every phase a few microseconds of
// dependent loads), the ticket chain of the task engine (task slot -> group
// slot -> instance total on the last warp -> controller) is most of a phase.
// This form (options.persistent = 2, B == 1) keeps the tasks but assigns them
// statically (warp w takes tasks w, w + warps, ...), so each warp sums its
// lanes' compensated partials over all its tasks; the block reduces its warps
// in warp order and stores one partial per block; after the grid barrier
// EVERY block reduces the block partials in block order and runs the step
// controller on its own shared-memory copy of the instance state.  The copies
// stay identical (same data, same operations), so no broadcast and no extra
// barrier is needed; block 0 writes the state back when the launch ends.
// Deterministic; the sums are grouped differently from the task engine's, so
// the iterates agree with the other forms to rounding, not bit for bit.
constexpr int kSoloThreads = 640;  // 20 warps per SM at 96 registers (measured best of 640 / 768 / 1024)
// Automatic step form: the single-LP form when the matrix (both sides) takes
// at most this many bytes, half of the 129 MB L2 (measured per step: 80k
// nonzeros 30.9 -> 20.8 us, 1.1M nonzeros 46.1 -> 38.8 us).
constexpr double kSoloMaxBytes = 64.0 * 1024.0 * 1024.0;
// Segments per light task on such an LP (the others keep kTaskSegs): a task's
// lane groups walk its segments one pointer round trip per pass, so on an
// L2-resident LP the tasks of short segments (128 columns of one nonzero at
// 128 nonzeros per task) set a phase's slowest warp.  Single-LP persistent
// form, per step: refinery 24 periods 16.2 -> 14.7 us, 168 periods
// 28.0 -> 26.0 us (32 segments: 14.3 / 26.9 us).
constexpr int kSoloTaskSegs = 64;

template <int Q>
__device__ __forceinline__ void solo_block_partial(Acc (&q)[Q], float2* __restrict__ out, Acc* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    warp_reduce_acc<Q>(q, 0u);
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < Q; ++i) sh[warp * Q + i] = q[i];
    __syncthreads();
    if (warp == 0) {
        Acc v[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            v[i].reset();
            if (lane < nwarps) v[i] = sh[lane * Q + i];
        }
        warp_reduce_acc<Q>(v, 0u);
        if (lane == 0)
#pragma unroll
            for (int i = 0; i < Q; ++i) out[i] = make_float2(v[i].s, v[i].c);
    }
}

// Totals of the P block partials (every block computes the same values);
// valid in thread 0.
template <int Q>
__device__ __forceinline__ void solo_grid_total(const float2* __restrict__ part, int P, double (&tot)[Q], Acc* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    Acc v[Q];
#pragma unroll
    for (int i = 0; i < Q; ++i) v[i].reset();
    for (int b = threadIdx.x; b < P; b += blockDim.x)
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const float2 w = __ldcg(part + (size_t)b * Q + i);
            Acc a;
            a.s = w.x;
            a.c = w.y;
            v[i] = acc_plus(v[i], a);
        }
    warp_reduce_acc<Q>(v, 0u);
    __syncthreads();  // sh is free again (the block partial is stored)
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < Q; ++i) sh[warp * Q + i] = v[i];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            v[i].reset();
            if (lane < nwarps) v[i] = sh[lane * Q + i];
        }
        warp_reduce_acc<Q>(v, 0u);
#pragma unroll
        for (int i = 0; i < Q; ++i) tot[i] = (double)v[i].s + (double)v[i].c;
    }
}

// This warp's static share of a side's tasks with epilogue `epi`; the lanes'
// partials (over all the warp's tasks) end in q.
template <int Q, class Epi>
__device__ __forceinline__ void solo_side(const Side& side, const Inst& S, Epi& epi, Acc (&q)[Q]) {
    const int nw = gridDim.x * (blockDim.x >> 5);
    const int lmax = side.light_max[0];
    epi.begin(S);
    for (int ti = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); ti < side.ntasks; ti += nw) {
        const Task t = side.tasks[ti];
        if (S.refine)
            run_any_task<1, true>(side, t, lmax, epi);
        else
            run_any_task<1, false>(side, t, lmax, epi);
    }
    epi.values(q);
}

// The single-LP form needs two grid barriers per step, not three: the
// primal step x' = clip(x - tau (c + K^T y), l, u) is not written by an
// elementwise phase before K x' gathers it, but computed by the gathering lane
// from a packed record per column, pack[j] = {x_j, c_j + (K^T y)_j, l_j, u_j}
// (one 16-byte load, the same L2 sector count as a float gather), with the
// same operations as the elementwise pass, so every lane gets the same x'_j.
// The column owner of the K^T y' phase computes x'_j the same way, stores it
// with the new K^T y' and the record of the next step (pack buffers follow the
// instance's `cur`); the pending average updates move to the owners (rows in
// K x', columns in K^T y').
__device__ __forceinline__ float4 ld_pack(const float4* p) {
    float4 v;
    asm volatile("ld.global.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
    return v;
}

__device__ __forceinline__ float primal_from_pack(const float4& r, float tau) {
    return fminf(fmaxf(fmaf(-tau, r.y, r.x), r.z), r.w);
}

struct DualStepEpiPacked : DualStepEpi {
    static constexpr bool kPackedX = true;
    const float4* pack_base;  // [2 N] records, one buffer per `cur`
    int ncols;                // N, columns of the whole batch
    const float4* pack;       // records of the instance's current point
    float tau, w;             // the primal step size and average weight, as step_scalars computes them
    int avg;
    int preset;               // 1: tau, w, avg were set by the caller (no FP64 division per warp)
    __device__ void begin(const Inst& S) {
        DualStepEpi::begin(S);
        if (!preset) {
            const StepScalars sc = step_scalars(S);
            tau = sc.tau;
            w = sc.w;
            avg = sc.avg;
        }
        pack = pack_base + (size_t)S.cur * ncols;
    }
    __device__ float gather_x(int j) const { return primal_from_pack(ld_pack(pack + j), tau); }
    __device__ void apply(int i, const SegDot<1>& d, const Pre& p) {
        if (avg) V.y_acc[i] = ff_axpy(V.y_acc[i], w, p.y);
        DualStepEpi::apply(i, d, p);
    }
};

// COHERENT: y' was written inside the same launch (the persistent form).
template <bool COHERENT>
struct KtyStepEpiPacked {
    static constexpr bool kCoherent = COHERENT;
    Vecs V;
    float4* pack_base;
    int ncols;
    const float4* pack;  // records of the current point
    float4* pack_next;   // records of the candidate point (the other buffer)
    const float *yg, *kty;
    float *xn, *ktyn;
    float tau, w;
    int avg;
    int preset;  // 1: tau, w, avg were set by the caller
    Acc inter, dx2;
    struct Pre { float4 r; float kty, c; };
    __device__ Pre pre(int j) const { return Pre{ld_pack(pack + j), kty[j], V.c[j]}; }
    __device__ void begin(const Inst& S) {
        if (!preset) {
            const StepScalars sc = step_scalars(S);
            tau = sc.tau;
            w = sc.w;
            avg = sc.avg;
        }
        pack = pack_base + (size_t)S.cur * ncols;
        pack_next = pack_base + (size_t)(S.cur ^ 1) * ncols;
        yg = pick(V.y0, V.y1, S.cur ^ 1);
        kty = pick(V.kty0, V.kty1, S.cur);
        ktyn = pick(V.kty0, V.kty1, S.cur ^ 1);
        xn = pick(V.x0, V.x1, S.cur ^ 1);
    }
    __device__ const float* gather(int) const { return yg; }
    __device__ void apply(int j, const SegDot<1>& d, const Pre& p) {
        const float k = d.f(0);
        const float x = p.r.x, xp = primal_from_pack(p.r, tau);
        if (avg) V.x_acc[j] = ff_axpy(V.x_acc[j], w, x);
        xn[j] = xp;
        ktyn[j] = k;
        pack_next[j] = make_float4(xp, p.c + k, p.r.z, p.r.w);
        const float dx = xp - x;
        inter.add(dx * (k - p.kty));
        dx2.add(dx * dx);
    }
    __device__ void values(Acc (&q)[2]) {
        q[0] = inter;
        q[1] = dx2;
        inter.reset();
        dx2.reset();
    }
    // the instance's step-size controller (task engine; the single-LP form runs
    // it itself after its grid reduction)
    __device__ void finish(Inst& S, const double* tot) { step_controller(S, tot[1], tot[0]); }
};

// Kernel-per-phase packed steps (options.packed): two kernels per step, the
// elementwise primal pass folded into them as in the single-LP form.  Same
// operations on the same values as the three-kernel step, so the iterates are
// bit-identical; the step moves the x' / average traffic of the elementwise
// pass into the two SpMV kernels.  Measured slower than the three kernels on
// bandwidth-bound LPs (a 16-byte record per gathered column costs more than
// the elementwise pass saves), so it is an option, off by default.
__global__ void __launch_bounds__(kThreads, 4)
    k_step_dual_packed(int B, Side rows, Vecs V, Inst* __restrict__ st, const float4* __restrict__ pack, int N) {
    chain_wait();
    step_schedule_pows(B, st, V);
    DualStepEpiPacked epi{{V}, pack, N};
    spmv_engine<1, true, 1>(rows, st, epi, 0u);
}

__global__ void __launch_bounds__(kThreads, 4) k_step_kty_packed(Side cols, Vecs V, Inst* __restrict__ st, float4* pack,
                                                                 int N) {
    chain_wait();
    KtyStepEpiPacked<false> epi{V, pack, N};
    spmv_engine<1, true, 2>(cols, st, epi, 0u);
}

// Records of every running instance's current point (after an evaluation,
// which may restart an instance at its average point).
__global__ void __launch_bounds__(kThreads) k_pack(Chunks ch, Vecs V, Inst* __restrict__ st, float4* pack, int N) {
    for_each_element(ch, st, step_scalars, [&](bool is_col, const StepScalars& S, int r) {
        if (!is_col) return;
        const float x = pick(V.x0, V.x1, S.cur)[r];
        const float kt = pick(V.kty0, V.kty1, S.cur)[r];
        pack[(size_t)S.cur * N + r] = make_float4(x, V.c[r] + kt, V.l[r], V.u[r]);
    });
}

__global__ void __launch_bounds__(kSoloThreads, 1)
    k_solo_steps(int nsteps, int N, Side rows, Side cols, Vecs V, Inst* st, GridBar gb, float2* part, float4* pack) {
    __shared__ Inst S;
    __shared__ StepScalars sc;  // the step's FP32 scalars, one FP64 division per block per step
    __shared__ Acc red[(kSoloThreads / 32) * 3];
    if (ld_status(gb.status) != 0) return;
    if (threadIdx.x == 0) {
        S = st[0];
        sc = step_scalars(S);
        schedule_pows(S, V);
    }
    unsigned long long gen = grid_start(gb);
    __syncthreads();
    // Block partials [2][P][3] (dy2, inter, dx2), double-buffered by step: the
    // |dy|^2 partials of K x' are reduced together with the K^T y' partials
    // after the step's last barrier (the controller is their only reader), and
    // a block can be writing the next step's partials while a slower one still
    // reads these.
    const int P = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
    // records of the current point (the evaluation between launches may have
    // moved it: a restart to the average)
    {
        const int c = S.cur;
        const float* x = pick(V.x0, V.x1, c);
        const float* kt = pick(V.kty0, V.kty1, c);
        float4* pk = pack + (size_t)c * N;
        for (int j = tid; j < N; j += nthreads) pk[j] = make_float4(x[j], V.c[j] + kt[j], V.l[j], V.u[j]);
    }
    if (!grid_barrier(gb, gen)) return;
    for (int k = 0; k < nsteps && !S.done; ++k) {
        float2* pb = part + (size_t)(k & 1) * 3 * P;
        // K x' (x' computed by the gathering lanes) and the dual step; sum |dy|^2
        const StepScalars s = sc;
        {
            DualStepEpiPacked epi{{V}, pack, N, nullptr, s.tau, s.w, s.avg, 1};
            Acc q[1];
            solo_side<1>(rows, S, epi, q);
            solo_block_partial<1>(q, pb + 3 * blockIdx.x, red);
        }
        if (!grid_barrier(gb, gen)) return;
        // K^T y', x' stored by the column owners, the next records, step terms
        {
            KtyStepEpiPacked<true> epi{V, pack, N};
            epi.tau = s.tau;
            epi.w = s.w;
            epi.avg = s.avg;
            epi.preset = 1;
            Acc q[2];
            solo_side<2>(cols, S, epi, q);
            solo_block_partial<2>(q, pb + 3 * blockIdx.x + 1, red);
        }
        if (!grid_barrier(gb, gen)) return;
        {
            double tot[3];
            solo_grid_total<3>(pb, P, tot, red);
            if (threadIdx.x == 0) {
                S.dy2 = tot[0];
                step_controller(S, tot[2], tot[1]);
                sc = step_scalars(S);
                schedule_pows(S, V);  // the next attempt's step-size schedule factors
            }
            __syncthreads();
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) st[0] = S;
}

// Barrier self-test (sih_pdhg_check_grid_barrier): `rounds` grid barriers;
// with gb.expected above the grid no barrier completes and every block's
// bounded wait runs out.
__global__ void k_barrier_probe(GridBar gb, int rounds, unsigned* passed) {
    unsigned long long gen = grid_start(gb);
    for (int r = 0; r < rounds; ++r) {
        if (!grid_barrier(gb, gen)) return;
        if (threadIdx.x == 0) atomicAdd(passed, 1u);
    }
}

// ---------------------------------------------------------------- evaluation kernels
// Before an evaluation: applies a pending average update and refreshes the
// FP32 copies x_avg, y_avg that the evaluation gathers.
__global__ void __launch_bounds__(kThreads) k_flush_avg(Chunks ch, Vecs V, Inst* __restrict__ st) {
    for_each_element(ch, st, step_scalars, [&](bool is_col, const StepScalars& S, int r) {
        if (is_col) {
            float2 a = V.x_acc[r];
            if (S.avg) V.x_acc[r] = a = ff_axpy(a, S.w, pick(V.x0, V.x1, S.cur)[r]);
            V.x_avg[r] = __fadd_rn(a.x, a.y);
        } else {
            float2 a = V.y_acc[r];
            if (S.avg) V.y_acc[r] = a = ff_axpy(a, S.w, pick(V.y0, V.y1, S.cur)[r]);
            V.y_avg[r] = __fadd_rn(a.x, a.y);
        }
    });
}

// Row evaluation of both candidates (0 = current, 1 = average): primal
// residual of K x_c against the row bounds (scaled 2-norm^2 and original
// inf-norm), row part of the dual objective, |y_c - y_last|^2.
struct EvalRowsEpi {
    Vecs V;
    const float *xg[2], *yc;
    Acc p2[2], dterm[2], dyl2[2];
    float pinf[2];
    struct Pre { float rl, ru, dr, yc, ya, yl; };
    __device__ Pre pre(int i) const { return Pre{V.rl[i], V.ru[i], V.drow[i], yc[i], V.y_avg[i], V.y_last[i]}; }
    __device__ void begin(const Inst& S) {
        xg[0] = pick(V.x0, V.x1, S.cur);
        xg[1] = V.x_avg;
        yc = pick(V.y0, V.y1, S.cur);
    }
    __device__ const float* gather(int v) const { return xg[v]; }
    __device__ void apply(int i, const SegDot<2>& d, const Pre& p) {
        V.kx_eval[i] = d.f(1);
        const float yv[2] = {p.yc, p.ya};
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const float res = row_violation(d.s[c], d.e[c], p.rl, p.ru);
            p2[c].add(res * res);
            pinf[c] = fmaxf(pinf[c], res / p.dr);
            row_dual_term(dterm[c], yv[c], p.rl, p.ru);
            const float dy = yv[c] - p.yl;
            dyl2[c].add(dy * dy);
        }
    }
    __device__ void values(Acc (&q)[8]) {
        q[0] = p2[0];
        q[1] = p2[1];
        q[2].s = pinf[0];
        q[2].c = 0.f;
        q[3].s = pinf[1];
        q[3].c = 0.f;
        q[4] = dterm[0];
        q[5] = dterm[1];
        q[6] = dyl2[0];
        q[7] = dyl2[1];
        for (int c = 0; c < 2; ++c) {
            p2[c].reset();
            dterm[c].reset();
            dyl2[c].reset();
            pinf[c] = 0.f;
        }
    }
    __device__ void finish(Inst& S, const double* tot) {
        for (int k = 0; k < 8; ++k) S.row_eval[k] = tot[k];
    }
};

__global__ void __launch_bounds__(kThreads) k_eval_rows(Side rows, Vecs V, Inst* __restrict__ st) {
    EvalRowsEpi epi{V};
    spmv_engine<2, true, 8>(rows, st, epi, 0x0Cu);
}

// Restart / termination controller of one instance after an evaluation.
__device__ void eval_controller(Inst& S, const double* cq, unsigned* done_count) {
    const double* rq = S.row_eval;
    double kkt[2], relp[2], reld[2], relg[2];
    const bool have_avg = S.W > 0.0;
    for (int c = 0; c < 2; ++c) {
        const double pobj = cq[4 + c];
        const double dobj = rq[4 + c] + cq[6 + c];
        const double gap = fabs(pobj - dobj);
        relp[c] = rq[2 + c] / (1.0 + S.b_inf);
        reld[c] = cq[2 + c] / (1.0 + S.c_inf);
        relg[c] = gap / (1.0 + fabs(pobj) + fabs(dobj));
        kkt[c] = sqrt(S.omega * rq[0 + c] + cq[0 + c] / S.omega + gap * gap);
        S.pobj[c] = pobj;
        S.dobj[c] = dobj;
        S.rel_p[c] = relp[c];
        S.rel_d[c] = reld[c];
        S.rel_g[c] = relg[c];
    }
    if (!have_avg) kkt[1] = INFINITY;
    S.evals += 1;
    S.avg_pending = 0;
    S.restart_flag = 0;
    if (!(kkt[0] == kkt[0])) {
        S.done = 3;
        S.out_sel = 0;
        atomicAdd(done_count, 1u);
        return;
    }
    // termination: current first, then the average
    for (int c = 0; c < 2; ++c) {
        if (c == 1 && !have_avg) break;
        if (relp[c] <= S.tol_p && reld[c] <= S.tol_d && relg[c] <= S.tol_g) {
            S.done = 1;
            S.out_sel = c;
            atomicAdd(done_count, 1u);
            return;
        }
    }
    const int cand = kkt[1] < kkt[0] ? 1 : 0;
    if (S.attempts >= S.max_attempts) {
        S.done = 2;
        S.out_sel = cand;
        atomicAdd(done_count, 1u);
        return;
    }
    const double worst = fmax(relp[cand] / S.tol_p, fmax(reld[cand] / S.tol_d, relg[cand] / S.tol_g));
    if (S.compensated == 2 || (S.compensated == 1 && worst < 100.0)) S.refine = 1;
    const double kc = kkt[cand];
    if (S.evals == 1) {  // initial point: record it as the last restart point
        S.kkt_last = kc;
        S.kkt_prev = kc;
        S.restart_flag = 1;
        return;
    }
    if (!S.enable_restart) return;
    const bool restart = kc <= S.beta_suff * S.kkt_last ||
                         (kc <= S.beta_nec * S.kkt_last && kc > S.kkt_prev) ||
                         (double)S.since_restart >= S.beta_art * (double)S.steps;
    S.kkt_prev = kc;
    if (!restart) return;
    const double dxn = sqrt(S.col_eval_dist[cand]), dyn = sqrt(S.row_eval[6 + cand]);
    if (dxn > 1e-10 && dyn > 1e-10) {
        const double th = S.weight_smoothing;
        S.omega = exp(th * log(dyn / dxn) + (1.0 - th) * log(S.omega));
    }
    S.kkt_last = kc;
    S.restart_flag = cand == 1 ? 2 : 1;
    S.restarts += 1;
    S.since_restart = 0;
    S.W = 0.0;
}

// Column evaluation of both candidates: reduced cost lambda = c + K^T y_c,
// dual residual (the parts no finite bound carries; scaled 2-norm^2 and
// original inf-norm), primal objective, column part of the dual objective,
// |x_c - x_last|^2.  The warp completing an instance runs its controller.
struct EvalColsEpi {
    Vecs V;
    unsigned* done_count;
    const float *yg[2], *xc;
    Acc d2[2], pobj[2], dterm[2], dxl2[2];
    float dinf[2];
    struct Pre { float c, l, u, dc, xc, xa, xl; };
    __device__ Pre pre(int j) const {
        return Pre{V.c[j], V.l[j], V.u[j], V.dcol[j], xc[j], V.x_avg[j], V.x_last[j]};
    }
    __device__ void begin(const Inst& S) {
        yg[0] = pick(V.y0, V.y1, S.cur);
        yg[1] = V.y_avg;
        xc = pick(V.x0, V.x1, S.cur);
    }
    __device__ const float* gather(int v) const { return yg[v]; }
    __device__ void apply(int j, const SegDot<2>& d, const Pre& p) {
        V.kty_eval[j] = d.f(1);
        const float xv[2] = {p.xc, p.xa};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            float h, lo;  // lambda = c + (s + e) as the float-float h + lo
            two_sum(p.c, d.s[k], h, lo);
            lo = __fadd_rn(lo, d.e[k]);
            const float lam = __fadd_rn(h, lo);
            float rd = 0.f;
            if (lam > 0.f) {
                if (fin(p.l)) { dterm[k].add_prod(h, p.l); dterm[k].add(lo * p.l); } else rd = lam;
            } else if (lam < 0.f) {
                if (fin(p.u)) { dterm[k].add_prod(h, p.u); dterm[k].add(lo * p.u); } else rd = -lam;
            }
            d2[k].add(rd * rd);
            dinf[k] = fmaxf(dinf[k], rd / p.dc);
            pobj[k].add_prod(p.c, xv[k]);
            const float dx = xv[k] - p.xl;
            dxl2[k].add(dx * dx);
        }
    }
    __device__ void values(Acc (&q)[10]) {
        q[0] = d2[0];
        q[1] = d2[1];
        q[2].s = dinf[0];
        q[2].c = 0.f;
        q[3].s = dinf[1];
        q[3].c = 0.f;
        q[4] = pobj[0];
        q[5] = pobj[1];
        q[6] = dterm[0];
        q[7] = dterm[1];
        q[8] = dxl2[0];
        q[9] = dxl2[1];
        for (int k = 0; k < 2; ++k) {
            d2[k].reset();
            pobj[k].reset();
            dterm[k].reset();
            dxl2[k].reset();
            dinf[k] = 0.f;
        }
    }
    __device__ void finish(Inst& S, const double* tot) {
        S.col_eval_dist[0] = tot[8];
        S.col_eval_dist[1] = tot[9];
        eval_controller(S, tot, done_count);
    }
};

__global__ void __launch_bounds__(kThreads) k_eval_cols(Side cols, Vecs V, Inst* __restrict__ st,
                                                        unsigned* done_count) {
    EvalColsEpi epi{V, done_count};
    spmv_engine<2, true, 10>(cols, st, epi, 0x0Cu);
}

// Applies a restart decided by the evaluation: restart to the average copies
// the average point (and its products from the evaluation) into the current
// buffers; either restart makes the new current point the last restart point
// and the start of the next average.
__global__ void __launch_bounds__(kThreads) k_restart(Chunks ch, Vecs V, Inst* __restrict__ st) {
    for_each_element(ch, st, step_scalars, [&](bool is_col, const StepScalars& S, int r) {
        const int flag = S.flag;
        if (flag == 0) return;
        if (is_col) {
            float* x = pick(V.x0, V.x1, S.cur);
            if (flag == 2) {
                x[r] = V.x_avg[r];
                pick(V.kty0, V.kty1, S.cur)[r] = V.kty_eval[r];
            }
            V.x_last[r] = x[r];
            V.x_acc[r] = make_float2(x[r], 0.f);
        } else {
            float* y = pick(V.y0, V.y1, S.cur);
            if (flag == 2) {
                y[r] = V.y_avg[r];
                pick(V.kx0, V.kx1, S.cur)[r] = V.kx_eval[r];
            }
            V.y_last[r] = y[r];
            V.y_acc[r] = make_float2(y[r], 0.f);
        }
    });
}

// ---------------------------------------------------------------- setup kernels
// Setup passes over every segment of a side, through its tasks: a light
// task's lanes take one segment each (segments longer than light_max are
// skipped), a list task's warp takes its listed segments one by one.  Every
// segment is visited exactly once, long ones by a whole warp.
template <class Light, class Long>
__device__ __forceinline__ void for_each_segment_tasks(const Side& sd, Light&& light, Long&& heavy) {
    const int lane = threadIdx.x & 31;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int ti = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); ti < sd.ntasks; ti += nw) {
        const Task t = sd.tasks[ti];
        if (t.flags & kTaskList) {
            for (int h = t.seg_begin; h < t.seg_end; ++h) heavy(sd.list_idx[h], lane);
        } else {
            const int lmax = sd.light_max[t.inst];
            for (int r = t.seg_begin + lane; r < t.seg_end; r += 32) {
                const int b = sd.A.ptr[r], e = sd.A.ptr[r + 1];
                if (e - b <= lmax) light(r, b, e);
            }
        }
    }
}

// Per-segment max |a| (mode 0) or sum |a| (mode 1) -> scale 1/sqrt(.) (1 if 0).
// Sums keep the entry order (one thread per segment).
__global__ void k_seg_scale(Side sd, int mode, float* __restrict__ scale) {
    const SegMatrix A = sd.A;
    auto fin_scale = [](float acc) { return acc > 0.f ? 1.0f / sqrtf(acc) : 1.0f; };
    for_each_segment_tasks(
        sd,
        [&](int r, int b, int e) {
            float acc = 0.f;
            for (int k = b; k < e; ++k) {
                const float a = fabsf(__int_as_float(A.pairs[k].y));
                acc = mode == 0 ? fmaxf(acc, a) : acc + a;
            }
            scale[r] = fin_scale(acc);
        },
        [&](int r, int lane) {
            const int b = A.ptr[r], e = A.ptr[r + 1];
            float acc = 0.f;
            if (mode == 0) {
                for (int k = b + lane; k < e; k += 32) acc = fmaxf(acc, fabsf(__int_as_float(A.pairs[k].y)));
                acc = warp_max(acc);
            } else if (lane == 0) {
                for (int k = b; k < e; ++k) acc += fabsf(__int_as_float(A.pairs[k].y));
            }
            if (lane == 0) scale[r] = fin_scale(acc);
        });
}

// a <- a * own[seg] * other[index] for every entry of one side.
__global__ void k_scale_entries(Side sd, const float* __restrict__ own, const float* __restrict__ other) {
    int2* pairs = const_cast<int2*>(sd.A.pairs);
    auto upd = [&](int k, float fs) {
        int2 p = pairs[k];
        p.y = __float_as_int(__int_as_float(p.y) * fs * other[p.x]);
        pairs[k] = p;
    };
    for_each_segment_tasks(
        sd,
        [&](int r, int b, int e) {
            const float fs = own[r];
            for (int k = b; k < e; ++k) upd(k, fs);
        },
        [&](int r, int lane) {
            const float fs = own[r];
            for (int k = sd.A.ptr[r] + lane; k < sd.A.ptr[r + 1]; k += 32) upd(k, fs);
        });
}

__global__ void k_mul_inplace(int n, float* __restrict__ acc, const float* __restrict__ f) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc[i] *= f[i];
}

// Scaled data: c~ = c d, l~ = l / d, u~ = u / d; rl~ = rl r, ru~ = ru r.
__global__ void k_scale_vectors(int N, int M, float* c, float* l, float* u, const float* dcol, float* rl, float* ru,
                                const float* drow) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
        c[j] *= dcol[j];
        l[j] /= dcol[j];
        u[j] /= dcol[j];
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        rl[i] *= drow[i];
        ru[i] *= drow[i];
    }
}

// Per-instance statistics of the scaled problem for the initial step size and
// primal weight: rows give max |a~| and |b~|^2, columns give |c~|^2.  Light
// tasks cover every segment (|b~|^2, |c~|^2) and the light segments' entries,
// list tasks the long segments' entries.
template <bool ROWS>
struct StatsEpi {
    Vecs V;
    float amax;
    Acc sq;
    __device__ void values(Acc (&q)[2]) {
        q[0].s = amax;
        q[0].c = 0.f;
        q[1] = sq;
        amax = 0.f;
        sq.reset();
    }
    __device__ void finish(Inst& S, const double* tot) {
        if (ROWS) {
            S.kmax = tot[0];
            S.b2 = tot[1];
        } else {
            S.c2 = tot[1];
        }
    }
};

template <bool ROWS>
__device__ void init_stats_side(const Side& sd, const Vecs& V, Inst* st) {
    const int lane = threadIdx.x & 31;
    StatsEpi<ROWS> epi{V, 0.f, Acc{}};
    task_loop<2>(sd, st, epi, 0x1u, [](const Inst&, int) {}, [&](const Task& t, const Inst&) {
        if (t.flags & kTaskList) {  // max |a| over the listed (long) segments
            for (int h = t.seg_begin; h < t.seg_end; ++h) {
                const int r = sd.list_idx[h];
                for (int k = sd.A.ptr[r] + lane; k < sd.A.ptr[r + 1]; k += 32)
                    epi.amax = fmaxf(epi.amax, fabsf(__int_as_float(sd.A.pairs[k].y)));
            }
            return;
        }
        const int lmax = sd.light_max[t.inst];
        for (int r = t.seg_begin + lane; r < t.seg_end; r += 32) {  // max |a| over the light segments
            const int b = sd.A.ptr[r], e = sd.A.ptr[r + 1];
            if (e - b > lmax) continue;
            for (int k = b; k < e; ++k) epi.amax = fmaxf(epi.amax, fabsf(__int_as_float(sd.A.pairs[k].y)));
        }
        for (int s = t.seg_begin + lane; s < t.seg_end; s += 32) {
            if (ROWS) {
                const float lo = V.rl[s], hi = V.ru[s];
                const float b = fin(lo) ? lo : (fin(hi) ? hi : 0.f);
                epi.sq.add_prod(b, b);
            } else {
                epi.sq.add_prod(V.c[s], V.c[s]);
            }
        }
    });
}

__global__ void __launch_bounds__(kThreads) k_init_stats_rows(Side rows, Vecs V, Inst* __restrict__ st) {
    init_stats_side<true>(rows, V, st);
}
__global__ void __launch_bounds__(kThreads) k_init_stats_cols(Side cols, Vecs V, Inst* __restrict__ st) {
    init_stats_side<false>(cols, V, st);
}

__global__ void k_init_controller(int B, Inst* st, double step_scale) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    Inst& S = st[b];
    S.eta = S.kmax > 0.0 ? step_scale / S.kmax : 1.0;
    const double cn = sqrt(S.c2), bn = sqrt(S.b2);
    S.omega = S.omega_start > 0.0 ? S.omega_start : ((cn > 1e-10 && bn > 1e-10) ? cn / bn : 1.0);
}

// Initial point x = clip(0, l~, u~) in both buffers, as the average and as the
// last restart point; y = 0 everywhere; K^T y = 0.
__global__ void k_init_point(int N, int M, Vecs V) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
        const float x = fminf(fmaxf(0.0f, V.l[j]), V.u[j]);
        V.x0[j] = x;
        V.x1[j] = x;
        V.x_avg[j] = x;
        V.x_last[j] = x;
        V.x_acc[j] = make_float2(x, 0.f);
        V.kty0[j] = 0.f;
        V.kty1[j] = 0.f;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
        V.y0[i] = 0.f;
        V.y1[i] = 0.f;
        V.y_avg[i] = 0.f;
        V.y_last[i] = 0.f;
        V.y_acc[i] = make_float2(0.f, 0.f);
    }
}

// Warm start of one instance: staged unscaled x (columns [c0, c1)) and y (rows
// [r0, r1)) in the x1 / y1 buffers become the scaled start point
// x~ = clip(x / dcol, l~, u~), y~ = y / drow, in every copy the initial point has.
__global__ void k_apply_start(int c0, int c1, int r0, int r1, Vecs V) {
    for (int j = c0 + blockIdx.x * blockDim.x + threadIdx.x; j < c1; j += gridDim.x * blockDim.x) {
        const float x = fminf(fmaxf(V.x1[j] / V.dcol[j], V.l[j]), V.u[j]);
        V.x0[j] = x;
        V.x1[j] = x;
        V.x_avg[j] = x;
        V.x_last[j] = x;
        V.x_acc[j] = make_float2(x, 0.f);
    }
    for (int i = r0 + blockIdx.x * blockDim.x + threadIdx.x; i < r1; i += gridDim.x * blockDim.x) {
        const float y = V.y1[i] / V.drow[i];
        V.y0[i] = y;
        V.y1[i] = y;
        V.y_avg[i] = y;
        V.y_last[i] = y;
        V.y_acc[i] = make_float2(y, 0.f);
    }
}

// y = K x for the initial point (row tasks, plain FP32 sums).
struct StoreEpi {
    const float* vec;
    float* out;
    struct Pre {};
    __device__ Pre pre(int) const { return Pre{}; }
    __device__ void begin(const Inst&) {}
    __device__ const float* gather(int) const { return vec; }
    __device__ void apply(int i, const SegDot<1>& d, const Pre&) { out[i] = d.s[0]; }
    __device__ void values(Acc (&q)[1]) { q[0].reset(); }
    __device__ void finish(Inst&, const double*) {}
};

__global__ void __launch_bounds__(kThreads) k_spmv_store(Side side, Inst* __restrict__ st, const float* __restrict__ vec,
                                                         float* __restrict__ out) {
    StoreEpi epi{vec, out};
    spmv_engine<1, false, 1>(side, st, epi, 0u);
}

// ---------------------------------------------------------------- active lists
// After an evaluation: the tasks (both sides) and element chunks of the
// instances still running, in instance order.  One block computes the
// per-instance offsets (prefix sums over the instances) ...
__global__ void k_compact_offsets(int B, const Inst* __restrict__ st, const int* __restrict__ rt,
                                  const int* __restrict__ ct, const int* __restrict__ hb, int* off, int* counts,
                                  unsigned* row_counter, unsigned* col_counter) {
    __shared__ int carry[3];
    __shared__ int wsum[3][32];
    if (threadIdx.x < 3) carry[threadIdx.x] = 0;
    if (threadIdx.x == 0) {  // task counters restart with the new lists
        *row_counter = 0u;
        *col_counter = 0u;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int base = 0; base < B; base += blockDim.x) {
        const int b = base + threadIdx.x;
        int v[3] = {0, 0, 0};
        if (b < B && !st[b].done) {
            v[0] = rt[b + 1] - rt[b];
            v[1] = ct[b + 1] - ct[b];
            v[2] = hb[b + 1] - hb[b];
        }
        int incl[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            int x = v[k];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULL_MASK, x, o);
                if (lane >= o) x += y;
            }
            incl[k] = x;
            if (lane == 31) wsum[k][warp] = x;
        }
        __syncthreads();
        if (b < B) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                int before = carry[k];
                for (int w = 0; w < warp; ++w) before += wsum[k][w];
                off[k * B + b] = before + incl[k] - v[k];
            }
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            int t = 0;
            for (int w = 0; w < nwarps; ++w) t += wsum[threadIdx.x][w];
            carry[threadIdx.x] += t;
        }
        __syncthreads();
    }
    if (threadIdx.x < 3) counts[threadIdx.x] = carry[threadIdx.x];
}

// ... and the grid scatters the entries of the running instances.
__global__ void k_compact_fill(int B, const Inst* __restrict__ st, Side rows, Side cols, Chunks ch,
                               const int* __restrict__ off) {
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows.ntasks; i += stride) {
        const int b = rows.tasks[i].inst;
        if (!st[b].done) rows.active[off[b] + i - rows.inst_task_begin[b]] = i;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cols.ntasks; i += stride) {
        const int b = cols.tasks[i].inst;
        if (!st[b].done) cols.active[off[B + b] + i - cols.inst_task_begin[b]] = i;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ch.n; i += stride) {
        const int b = ch.chunks[i].z;
        if (!st[b].done) ch.active[off[2 * B + b] + i - ch.inst_begin[b]] = i;
    }
}

// ---------------------------------------------------------------- host: schedule
// Shortest run of long segments that a light task skips instead of walking:
// one pass of 1-lane groups.
constexpr int kSkipRun = 32;

static int pow2_floor(int v) {
    int p = 1;
    while (p * 2 <= v) p *= 2;
    return p;
}

void make_schedule(const std::vector<int>& ptr, const std::vector<int>& inst_off, int task_nnz, SideSchedule& out,
                   int light_lanes, int max_segs) {
    if (light_lanes > 0) light_lanes = std::min(32, pow2_floor(light_lanes));
    max_segs = std::max(1, std::min(kTaskSegs, max_segs));
    const int B = (int)inst_off.size() - 1;
    out = SideSchedule{};
    out.light_max.assign(B, 0);
    for (int b = 0; b < B; ++b) {
        const int s0 = inst_off[b], s1 = inst_off[b + 1];
        const long long nnz = ptr[s1] - ptr[s0];
        const int nseg = s1 - s0;
        const int mean = nseg > 0 ? (int)((nnz + nseg - 1) / nseg) : 1;
        // light segments: up to two load batches per lane of the instance's mean lane group
        const int L0 = std::max(1, std::min(32, pow2_floor(std::max(1, mean / kBatch))));
        const int lmax = std::max(2 * kBatch * L0, 8);
        out.light_max[b] = lmax;
        // light tasks: contiguous, at most task_nnz light nonzeros / max_segs
        // segments.  A light task does not start on a run of at least
        // kSkipRun long segments (the list tasks own those): after the
        // renumbering by length they are the instance's prefix, which the
        // first task would otherwise walk one pointer round trip per pass of
        // its lane groups (refinery LP with 168 periods: 1,344 long rows,
        // 6.5 us per A x' phase on that warp).  A shorter run is walked in the
        // task's first pass anyway and stays in it.
        int s = s0;
        while (s < s1) {
            int run = 0;
            while (s + run < s1 && ptr[s + run + 1] - ptr[s + run] > lmax) ++run;
            if (run >= kSkipRun) {
                s += run;
                continue;
            }
            int e = s;
            long long acc = 0;
            while (e < s1 && e - s < max_segs) {
                const int len = ptr[e + 1] - ptr[e];
                const long long add = len > lmax ? 0 : len;
                if (e > s && acc + add > task_nnz) break;
                acc += add;
                ++e;
            }
            const int nl = std::max(1, e - s);
            const int L = light_lanes > 0 ? light_lanes
                                          : std::max(1, std::min(32, pow2_floor(std::max(1, (int)(acc / nl) / kBatch))));
            out.tasks.push_back(Task{s, e, b, L << 8});
            s = e;
        }
        // list tasks: longer segments by length class (lmax, 2 lmax], (2 lmax, 4 lmax], ...,
        // lanes doubling per class; the last class (32 lanes) is open-ended.  One
        // bucketing pass, segments in index order inside each class.
        std::vector<std::pair<int, int>> classes;  // (lo, lanes)
        for (int lo = lmax, L = std::min(32, 2 * L0); lo < (1 << 30); lo *= 2, L = std::min(32, 2 * L)) {
            classes.push_back({lo, L});
            if (L == 32) break;
        }
        std::vector<std::vector<int>> bucket(classes.size());
        for (int r = s0; r < s1; ++r) {
            const int len = ptr[r + 1] - ptr[r];
            if (len <= lmax) continue;
            size_t k = 0;
            while (k + 1 < classes.size() && len > 2 * classes[k].first) ++k;
            if (len > classes[k].first) bucket[k].push_back(r);
        }
        for (size_t kc = 0; kc < classes.size(); ++kc) {
            const int L = classes[kc].second;
            const int hb = (int)out.list_idx.size();
            out.list_idx.insert(out.list_idx.end(), bucket[kc].begin(), bucket[kc].end());
            int h = hb;
            while (h < (int)out.list_idx.size()) {
                int e = h;
                long long acc = 0;
                while (e < (int)out.list_idx.size()) {
                    const int len = ptr[out.list_idx[e] + 1] - ptr[out.list_idx[e]];
                    if (e > h && acc + len > task_nnz) break;
                    acc += len;
                    ++e;
                }
                out.tasks.push_back(Task{h, e, b, kTaskList | (L << 8)});
                h = e;
            }
            if (L == 32) break;
        }
    }
    // reduction groups: at most kGroup consecutive tasks of one instance
    const int nt = (int)out.tasks.size();
    out.task_group.assign(nt, 0);
    out.inst_group_begin.assign(B + 1, 0);
    int t = 0;
    for (int b = 0; b < B; ++b) {
        out.inst_group_begin[b] = (int)out.group_begin.size();
        while (t < nt && out.tasks[t].inst == b) {
            const int g = (int)out.group_begin.size();
            out.group_begin.push_back(t);
            for (int k = 0; k < kGroup && t < nt && out.tasks[t].inst == b; ++k, ++t) out.task_group[t] = g;
        }
    }
    out.inst_group_begin[B] = (int)out.group_begin.size();
    out.group_begin.push_back(nt);
    out.inst_task_begin.assign(B + 1, nt);
    for (int k = nt - 1; k >= 0; --k) out.inst_task_begin[out.tasks[k].inst] = k;
    for (int b = B - 1; b >= 0; --b) out.inst_task_begin[b] = std::min(out.inst_task_begin[b], out.inst_task_begin[b + 1]);
}

// ---------------------------------------------------------------- host: solver
MixedSolver::~MixedSolver() {
    for (auto& g : graphs_)
        if (g) cudaGraphExecDestroy(g);
    if (ev_start_) cudaEventDestroy(ev_start_);
    if (ev_stop_) cudaEventDestroy(ev_stop_);
    if (stream_) cudaStreamDestroy(stream_);
}

// Renumbered pairs of one side: segment s (new order) takes the entries of
// its source segment (src[s].x = first source entry, same length) with the
// other side's indices mapped through inv (src[s].y = that side's instance
// offset).  One warp per segment, lanes over its entries.
__global__ void k_renumber_pairs(int nseg, const int* __restrict__ ptr, const int2* __restrict__ src,
                                 const int2* __restrict__ in, const int* __restrict__ inv, int2* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int sg = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); sg < nseg; sg += nw) {
        const int b = ptr[sg], len = ptr[sg + 1] - b;
        const int2 sc = src[sg];
        for (int k = lane; k < len; k += 32) {
            const int2 p = in[sc.x + k];
            out[b + k] = make_int2(inv[sc.y + p.x], p.y);
        }
    }
}

// Stable order of `cnt` segments by descending length (counting sort); the
// identity without `reorder`.
static void order_by_length(const int* ptr, int cnt, bool reorder, int* perm) {
    if (!reorder || cnt <= 1) {
        for (int k = 0; k < cnt; ++k) perm[k] = k;
        return;
    }
    int maxlen = 0;
    for (int k = 0; k < cnt; ++k) maxlen = std::max(maxlen, ptr[k + 1] - ptr[k]);
    std::vector<int> start((size_t)maxlen + 2, 0);
    for (int k = 0; k < cnt; ++k) start[maxlen - (ptr[k + 1] - ptr[k]) + 1]++;
    for (int v = 0; v <= maxlen; ++v) start[v + 1] += start[v];
    for (int k = 0; k < cnt; ++k) perm[start[maxlen - (ptr[k + 1] - ptr[k])]++] = k;
}

static int upload(DevMem& d, const void* h, size_t bytes, cudaStream_t s) {
    SIHG_TRY(d.alloc(bytes));
    if (bytes) SIHG_CUDA(cudaMemcpyAsync(d.as<void>(), h, bytes, cudaMemcpyHostToDevice, s));
    return SIH_PDHG_OK;
}

// One LP whose matrix (both sides, 16 bytes per nonzero) fits in half of L2.
bool MixedSolver::latency_bound() const { return B_ == 1 && 16.0 * (double)nnz_ <= kSoloMaxBytes; }

// Tasks, reduction groups, tickets, element chunks and active lists for SpMV
// tasks of about `task_nnz` nonzeros (rebuilt by the autotuner).
int MixedSolver::build_schedules(int task_nnz) {
    task_nnz_ = task_nnz;
    if (graphs_[0]) {  // the recorded graph holds the old schedules
        cudaGraphExecDestroy(graphs_[0]);
        graphs_[0] = nullptr;
    }
    SIHG_TRY(layout_.build(h_csr_ptr_, h_csc_ptr_, row_off_, col_off_,
                           SegMatrix{M_, csr_ptr_.as<int>(), csr_pairs_.as<int2>()},
                           SegMatrix{N_, csc_ptr_.as<int>(), csc_pairs_.as<int2>()}, task_nnz_, false, stream_,
                           lanes_r_, lanes_c_, latency_bound() ? kSoloTaskSegs : kTaskSegs));
    rows_ = layout_.rows;
    cols_ = layout_.cols;
    chunks_all_ = layout_.chunks;
    return SIH_PDHG_OK;
}

int MixedSolver::setup(const std::vector<const HostProblem*>& probs, const sih_pdhg_config& cfg,
                       const sih_pdhg_options& opts) {
    probs_ = probs;
    cfg_ = cfg;
    opts_ = opts;
    B_ = (int)probs.size();
    int dev = 0;
    SIHG_CUDA(cudaGetDevice(&dev));
    SIHG_CUDA(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, dev));
    SIHG_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    SIHG_CUDA(cudaEventCreate(&ev_start_));
    SIHG_CUDA(cudaEventCreate(&ev_stop_));
    cudaStream_t s = stream_;
    auto t_last = std::chrono::steady_clock::now();
    auto phase = [&](const char* what) {  // options.verbose: host time of each set-up phase
        if (!opts.verbose) return;
        cudaStreamSynchronize(s);
        const auto t = std::chrono::steady_clock::now();
        std::fprintf(stderr, "sih_pdhg setup: %-18s %.4f s\n", what, std::chrono::duration<double>(t - t_last).count());
        t_last = t;
    };

    // ---- concatenate the instances (block-diagonal), global indices
    row_off_.assign(B_ + 1, 0);
    col_off_.assign(B_ + 1, 0);
    long long nnz = 0;
    for (int b = 0; b < B_; ++b) {
        row_off_[b + 1] = row_off_[b] + probs[b]->m;
        col_off_[b + 1] = col_off_[b] + probs[b]->n;
        nnz += probs[b]->nnz;
    }
    M_ = row_off_[B_];
    N_ = col_off_[B_];
    nnz_ = nnz;
    if ((long long)M_ >= INT32_MAX - 64 || (long long)N_ >= INT32_MAX - 64 || nnz >= INT32_MAX - 64)
        return fail(SIH_PDHG_ERR_UNSUPPORTED, "batch exceeds the 32-bit index layout");
    std::vector<int> csr_ptr((size_t)M_ + 1), csc_ptr((size_t)N_ + 1);
    std::vector<float> c(N_), l(N_), u(N_), rl(M_), ru(M_);
    // Renumbering inside each instance (opts.reorder): columns and rows by
    // descending length.  The entries that long segments share then sit in
    // few cache lines of the gathered vectors (for Zipf-like column lengths
    // most of A x's gathers hit an L1-sized prefix of x).  perm: new -> old,
    // local to the instance.
    col_perm_.assign(N_, 0);
    row_perm_.assign(M_, 0);
    std::vector<long long> k_off(B_ + 1, 0);
    for (int b = 0; b < B_; ++b) k_off[b + 1] = k_off[b] + probs[b]->nnz;
    const bool reorder = opts.reorder != 0;
    parallel_for_min(2 * (int64_t)B_, 1, [&](int64_t w0, int64_t w1) {
        for (int64_t w = w0; w < w1; ++w) {
            const int b = (int)(w >> 1);
            const HostProblem& p = *probs[b];
            const bool cols = (w & 1) == 0;
            const std::vector<int>& ptr = cols ? p.csc_ptr : p.csr_ptr;
            const int cnt = cols ? p.n : p.m;
            const int off = cols ? col_off_[b] : row_off_[b];
            int* perm = (cols ? col_perm_.data() : row_perm_.data()) + off;
            order_by_length(ptr.data(), cnt, reorder, perm);
            // pointers of the renumbered segments
            int* dst = (cols ? csc_ptr.data() : csr_ptr.data()) + off;
            long long acc = k_off[b];
            for (int k = 0; k < cnt; ++k) {
                dst[k] = (int)acc;
                acc += ptr[perm[k] + 1] - ptr[perm[k]];
            }
        }
    });
    csr_ptr[M_] = (int)nnz;
    csc_ptr[N_] = (int)nnz;
    // Per renumbered segment (columns, then rows): its first entry in the
    // pairs as uploaded (each instance's CSC / CSR in its original order) and
    // the other side's instance offset; inv: global original index -> global
    // new index (columns, then rows).  The device writes the renumbered pairs
    // (k_renumber_pairs), so the host work stays O(rows + columns).
    std::vector<int2> seg_src((size_t)N_ + M_);
    std::vector<int> inv((size_t)N_ + M_);
    struct Piece {
        int b, cols, k0, k1;
    };
    std::vector<Piece> pieces;
    for (int b = 0; b < B_; ++b)
        for (int side = 0; side < 2; ++side) {
            const int cnt = side == 0 ? probs[b]->n : probs[b]->m;
            for (int k0 = 0; k0 < cnt; k0 += 32768) pieces.push_back(Piece{b, side == 0, k0, std::min(cnt, k0 + 32768)});
        }
    // infinite bounds are +-inf (|v| >= 1e20 counts as infinite)
    auto inf_clean = [](double v) -> float {
        if (std::isinf(v) || std::fabs(v) >= 1e20) return v > 0 ? INFINITY : -INFINITY;
        return (float)v;
    };
    parallel_for_min((int64_t)pieces.size(), 1, [&](int64_t q0, int64_t q1) {
        for (int64_t q = q0; q < q1; ++q) {
            const Piece& pc = pieces[q];
            const HostProblem& p = *probs[pc.b];
            const int ro = row_off_[pc.b], co = col_off_[pc.b];
            const int kb = (int)k_off[pc.b];
            if (pc.cols) {
                for (int jn = pc.k0; jn < pc.k1; ++jn) {
                    const int j = col_perm_[co + jn];
                    inv[co + j] = co + jn;
                    seg_src[co + jn] = make_int2(kb + p.csc_ptr[j], ro);
                    c[co + jn] = p.c[j];
                    l[co + jn] = inf_clean(p.src->col_lower[j]);
                    u[co + jn] = inf_clean(p.src->col_upper[j]);
                }
            } else {
                for (int in = pc.k0; in < pc.k1; ++in) {
                    const int i = row_perm_[ro + in];
                    inv[N_ + ro + i] = ro + in;
                    seg_src[N_ + ro + in] = make_int2(kb + p.csr_ptr[i], co);
                    rl[ro + in] = inf_clean(p.src->row_lower[i]);
                    ru[ro + in] = inf_clean(p.src->row_upper[i]);
                }
            }
        }
    });
    phase("renumber");
    // ---- schedules (tasks and reduction groups per side, element chunks)
    int occ = 0;
    SIHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_step_dual, kThreads, 0));
    grid_ = std::max(1, sm_count_ * std::max(1, occ));
    int occ_e = 0;
    SIHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_e, k_step_primal, kThreads, 0));
    elem_grid_ = std::max(1, sm_count_ * std::max(1, occ_e));
    // default task size: about three tasks per resident warp, within [128, 2048]
    const long long warps = (long long)grid_ * (kThreads / 32);
    task_nnz_ = opts.tile_nnz > 0 ? opts.tile_nnz
                                  : (int)std::max(128LL, std::min(2048LL, nnz / std::max(1LL, 3 * warps)));
    task_nnz_ = std::max(32, std::min(1 << 20, task_nnz_));
    SIHG_TRY(upload(csr_ptr_, csr_ptr.data(), sizeof(int) * csr_ptr.size(), s));
    SIHG_TRY(upload(csc_ptr_, csc_ptr.data(), sizeof(int) * csc_ptr.size(), s));
    {
        // each instance's pairs as they are, then the renumbered sides
        DevMem src, segs, invd;
        const size_t nz = (size_t)std::max<long long>(1, nnz);
        SIHG_TRY(src.alloc(sizeof(Pair) * 2 * nz));
        Pair* s_csc = src.as<Pair>();
        Pair* s_csr = s_csc + nz;
        for (int b = 0; b < B_; ++b) {
            const size_t nb = (size_t)probs[b]->nnz;
            if (nb == 0) continue;
            SIHG_CUDA(cudaMemcpyAsync(s_csc + k_off[b], probs[b]->csc.data(), sizeof(Pair) * nb,
                                      cudaMemcpyHostToDevice, s));
            SIHG_CUDA(cudaMemcpyAsync(s_csr + k_off[b], probs[b]->csr.data(), sizeof(Pair) * nb,
                                      cudaMemcpyHostToDevice, s));
        }
        SIHG_TRY(upload(segs, seg_src.data(), sizeof(int2) * seg_src.size(), s));
        SIHG_TRY(upload(invd, inv.data(), sizeof(int) * inv.size(), s));
        SIHG_TRY(csc_pairs_.alloc(sizeof(Pair) * nz));
        SIHG_TRY(csr_pairs_.alloc(sizeof(Pair) * nz));
        const int g = sm_count_ * 8;
        k_renumber_pairs<<<g, 256, 0, s>>>(N_, csc_ptr_.as<int>(), segs.as<int2>(), (const int2*)s_csc,
                                           invd.as<int>() + N_, csc_pairs_.as<int2>());
        k_renumber_pairs<<<g, 256, 0, s>>>(M_, csr_ptr_.as<int>(), segs.as<int2>() + N_, (const int2*)s_csr,
                                           invd.as<int>(), csr_pairs_.as<int2>());
        SIHG_LAUNCH_CHECK();
        SIHG_CUDA(cudaStreamSynchronize(s));  // the staging buffers are released at scope end
    }
    h_csr_ptr_ = std::move(csr_ptr);
    h_csc_ptr_ = std::move(csc_ptr);
    lanes_r_ = opts.lanes_csr;
    lanes_c_ = opts.lanes_csc;
    SIHG_TRY(build_schedules(task_nnz_));
    SIHG_TRY(choose_staging());

    phase("schedules+upload");
    // ---- vectors: 11 column vectors, 10 row vectors (layout of Vecs) + float-float averages
    SIHG_TRY(colvec_.alloc(sizeof(float) * (size_t)N_ * 11));
    SIHG_TRY(rowvec_.alloc(sizeof(float) * (size_t)M_ * 10));
    SIHG_TRY(accvec_.alloc(sizeof(float2) * ((size_t)N_ + M_)));
    float* cv = colvec_.as<float>();
    float* rv = rowvec_.as<float>();
    auto C = [&](int k) { return cv + (size_t)k * N_; };
    auto R = [&](int k) { return rv + (size_t)k * M_; };
    V_ = Vecs{C(0), C(1), C(2), C(3), C(4), C(5), C(6), C(7), C(8), C(9), C(10),
              R(0), R(1), R(2), R(3), R(4), R(5), R(6), R(7), R(8), R(9),
              accvec_.as<float2>(), accvec_.as<float2>() + N_};
    SIHG_CUDA(cudaMemcpyAsync(C(0), c.data(), sizeof(float) * N_, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(C(1), l.data(), sizeof(float) * N_, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(C(2), u.data(), sizeof(float) * N_, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(R(0), rl.data(), sizeof(float) * M_, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(R(1), ru.data(), sizeof(float) * M_, cudaMemcpyHostToDevice, s));

    phase("vectors");
    // ---- scaling (Ruiz inf-norm passes, then Pock-Chambolle alpha = 1)
    std::vector<float> ones_c(N_, 1.0f), ones_r(M_, 1.0f);
    SIHG_CUDA(cudaMemcpyAsync(C(3), ones_c.data(), sizeof(float) * N_, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(R(2), ones_r.data(), sizeof(float) * M_, cudaMemcpyHostToDevice, s));
    DevMem tmp;
    SIHG_TRY(tmp.alloc(sizeof(float) * ((size_t)N_ + M_ + 8)));
    float* fc = tmp.as<float>();
    float* fr = fc + N_;
    const int g = sm_count_ * 8;
    auto scale_pass = [&](int mode) -> int {
        k_seg_scale<<<g, 256, 0, s>>>(cols_, mode, fc);
        k_seg_scale<<<g, 256, 0, s>>>(rows_, mode, fr);
        k_scale_entries<<<g, 256, 0, s>>>(rows_, fr, fc);
        k_scale_entries<<<g, 256, 0, s>>>(cols_, fc, fr);
        k_mul_inplace<<<g, 256, 0, s>>>(N_, C(3), fc);
        k_mul_inplace<<<g, 256, 0, s>>>(M_, R(2), fr);
        SIHG_LAUNCH_CHECK();
        return SIH_PDHG_OK;
    };
    for (int k = 0; k < opts.ruiz_iterations; ++k) SIHG_TRY(scale_pass(0));
    if (opts.pock_chambolle) SIHG_TRY(scale_pass(1));
    k_scale_vectors<<<g, 256, 0, s>>>(N_, M_, C(0), C(1), C(2), C(3), R(0), R(1), R(2));
    SIHG_LAUNCH_CHECK();
    SIHG_CUDA(cudaStreamSynchronize(s));  // tmp is released at scope end

    phase("scaling");
    // ---- per-instance state
    SIHG_TRY(state_.alloc(sizeof(Inst) * B_));
    SIHG_TRY(done_count_.alloc(sizeof(unsigned)));
    host_inst_.assign(B_, Inst{});
    for (int b = 0; b < B_; ++b) {
        Inst& S = host_inst_[b];
        std::memset(&S, 0, sizeof(Inst));
        const sih_pdhg_problem* p = probs[b]->src;
        double binf = 0.0, cinf = 0.0;
        for (int64_t i = 0; i < p->num_rows; ++i) {
            if (bound_is_finite(p->row_lower[i])) binf = std::max(binf, std::fabs(p->row_lower[i]));
            if (bound_is_finite(p->row_upper[i])) binf = std::max(binf, std::fabs(p->row_upper[i]));
        }
        for (int64_t j = 0; j < p->num_cols; ++j) cinf = std::max(cinf, std::fabs(p->c[j]));
        S.b_inf = binf;
        S.c_inf = cinf;
        S.tol_p = cfg.tol_primal;
        S.tol_d = cfg.tol_dual;
        S.tol_g = cfg.tol_gap;
        S.max_attempts = cfg.max_iterations;
        S.enable_restart = cfg.enable_restart ? 1 : 0;
        S.compensated = opts.compensated;
        S.refine = opts.compensated == 2 ? 1 : 0;
        S.beta_suff = opts.restart_sufficient;
        S.beta_nec = opts.restart_necessary;
        S.beta_art = opts.restart_artificial;
        S.weight_smoothing = opts.primal_weight_smoothing;
    }
    {
        const long long need = (long long)cfg.max_iterations + 3;
        const int n = (int)std::max(3LL, std::min<long long>(need, kPowTable));
        SIHG_TRY(pow_tab_.alloc(sizeof(double2) * (size_t)n));
        k_pow_table<<<std::max(1, std::min(sm_count_ * 4, (n + 255) / 256)), 256, 0, s>>>(n, pow_tab_.as<double2>());
        SIHG_LAUNCH_CHECK();
        V_.pow_tab = pow_tab_.as<double2>();
        V_.pow_n = n;
    }
    phase("state");
    SIHG_TRY(setup_persistent());
    SIHG_TRY(setup_packed());
    // autotune: 1 on, 0 off, < 0 automatic (on for batches)
    if (opts.autotune > 0 || (opts.autotune < 0 && B_ > 1)) SIHG_TRY(autotune());
    return SIH_PDHG_OK;
}

// Packed kernel-per-phase steps (options.packed, off by default: slower where
// measured); the single-LP persistent form always works on the records.
int MixedSolver::setup_packed() {
    packed_ = opts_.packed > 0 ? 1 : 0;
    if ((packed_ || B_ == 1) && pack_.bytes() < sizeof(float4) * 2 * (size_t)std::max(1, N_))
        SIHG_TRY(pack_.alloc(sizeof(float4) * 2 * (size_t)std::max(1, N_)));
    return SIH_PDHG_OK;
}

// Persistent step kernel: every block must be resident at once (a
// cooperative launch checks it), so the grid is the SM count times the
// kernel's occupancy; the barrier words are reset at the start of each run.
int MixedSolver::setup_persistent() {
    persistent_ = 0;
    grid_form1_ = grid_form2_ = 0;
    int dev = 0, coop = 0, occ = 0;
    SIHG_CUDA(cudaGetDevice(&dev));
    SIHG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (coop) {
        SIHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_steps_persistent, kThreads, 0));
        grid_form1_ = sm_count_ * occ;
        if (B_ == 1) {
            SIHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_solo_steps, kSoloThreads, 0));
            grid_form2_ = sm_count_ * occ;
        }
        SIHG_TRY(bar_.alloc(4 * sizeof(unsigned)));
        SIHG_TRY(part_.alloc(sizeof(float2) * 6 * (size_t)std::max(1, grid_form2_)));
    }
    int form = opts_.persistent;
    if (form < 0) {
        // automatic: the single-LP form for one LP whose matrix (both sides,
        // 16 bytes per nonzero) fits in half of L2: its steps are latency-bound
        form = latency_bound() ? 2 : 0;
    }
    if (form == 2 && B_ != 1) form = 1;  // the single-LP form needs one LP
    return set_form(form);
}

// Step form in use: 0 kernels per phase (graphs), 1 / 2 persistent.
int MixedSolver::set_form(int form) {
    if (form != 0 && (form == 1 ? grid_form1_ : grid_form2_) < 1) {
        if (opts_.persistent > 0)
            return fail(SIH_PDHG_ERR_UNSUPPORTED, "options.persistent: no cooperative launch of the step kernel here");
        form = 0;
    }
    persistent_ = form;
    pgrid_ = form == 1 ? grid_form1_ : (form == 2 ? grid_form2_ : 0);
    return SIH_PDHG_OK;
}

// Longest wait of one grid barrier of the persistent kernel.  A phase of the
// largest batch this engine holds takes milliseconds; a wait this long means
// a block stopped arriving.
constexpr double kBarrierLimitSec = 2.0;

// Barrier words: a 64-bit arrival counter, then the status word.
static GridBar make_bar(const DevMem& words, unsigned expected, double limit_sec) {
    unsigned long long* w = words.as<unsigned long long>();
    return GridBar{w, reinterpret_cast<int*>(w + 1), expected, (unsigned long long)(limit_sec * 1e9)};
}

// One cooperative launch of the persistent step kernel: `nsteps` steps.
int MixedSolver::launch_persistent(cudaStream_t s, int nsteps) {
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)pgrid_);
    cfg.blockDim = dim3((unsigned)kThreads);
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const GridBar gb = make_bar(bar_, (unsigned)pgrid_, kBarrierLimitSec);
    cudaError_t e;
    if (persistent_ == 2) {
        cfg.blockDim = dim3((unsigned)kSoloThreads);
        e = cudaLaunchKernelEx(&cfg, k_solo_steps, nsteps, N_, rows_, cols_, V_, state_.as<Inst>(), gb,
                               part_.as<float2>(), pack_.as<float4>());
    } else {
        e = cudaLaunchKernelEx(&cfg, k_steps_persistent, B_, nsteps, chunks_all_, rows_, cols_, V_,
                               state_.as<Inst>(), gb);
    }
    if (e == cudaErrorCooperativeLaunchTooLarge && opts_.persistent < 0) {
        // the device cannot hold the whole grid at once now (SMs taken by other
        // work, or a partitioned device): nothing was launched; with the step
        // form left to the engine, these and all later steps run as kernels per
        // phase instead
        (void)cudaGetLastError();
        SIHG_TRY(set_form(0));
        for (int k = 0; k < nsteps; ++k) SIHG_TRY(launch_step(s));
        return SIH_PDHG_OK;
    }
    if (e != cudaSuccess) return cuda_fail(e, "persistent step kernel launch", __FILE__, __LINE__);
    launches_ += 1;
    return SIH_PDHG_OK;
}

int check_grid_barrier(int blocks, int missing, int rounds, double limit_sec, int* timed_out, int* passed) {
    if (blocks < 1 || missing < 0 || rounds < 1 || !(limit_sec > 0.0) || limit_sec > 10.0)
        return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "grid barrier check: blocks >= 1, missing >= 0, rounds >= 1, "
                                                   "0 < limit_sec <= 10");
    int dev = 0, sms = 0, occ = 0;
    SIHG_CUDA(cudaGetDevice(&dev));
    SIHG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SIHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_barrier_probe, kThreads, 0));
    if (blocks > sms * occ) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "grid barrier check: more blocks than fit");
    DevMem words;
    SIHG_TRY(words.alloc(8 * sizeof(unsigned)));
    SIHG_CUDA(cudaMemset(words.as<void>(), 0, 8 * sizeof(unsigned)));
    const GridBar gb = make_bar(words, (unsigned)(blocks + missing), limit_sec);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3((unsigned)kThreads);
    cfg.attrs = at;
    cfg.numAttrs = 1;
    SIHG_CUDA(cudaLaunchKernelEx(&cfg, k_barrier_probe, gb, rounds, words.as<unsigned>() + 6));
    SIHG_CUDA(cudaDeviceSynchronize());
    unsigned h[8];
    SIHG_CUDA(cudaMemcpy(h, words.as<void>(), sizeof(h), cudaMemcpyDeviceToHost));
    if (timed_out) *timed_out = (int)h[2];
    if (passed) *passed = (int)(h[6] / (unsigned)blocks);
    return SIH_PDHG_OK;
}

// Launches a step kernel (which starts with chain_wait) with programmatic
// stream serialization.
template <class... P, class... A>
static cudaError_t launch_chained(void (*kernel)(P...), int grid, int block, size_t smem, cudaStream_t s,
                                  A... args) {
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

int MixedSolver::launch_step(cudaStream_t s) {
    Inst* st = state_.as<Inst>();
    if (!packed_) {
        launches_ += 1;
        SIHG_CUDA(launch_chained(k_step_primal, elem_grid_, kThreads, 0, s, B_, chunks_all_, V_, st));
    }
    SIHG_TRY(launch_step_spmvs(s, 1));
    SIHG_TRY(launch_step_spmvs(s, 2));
    SIHG_LAUNCH_CHECK();
    return SIH_PDHG_OK;
}

// One of the step SpMVs (which = 1: K x' with the dual update, 2: K^T y' with
// the step-size controller), staged when choose_staging picked a prefix.
int MixedSolver::launch_step_spmvs(cudaStream_t s, int which) {
    Inst* st = state_.as<Inst>();
    launches_ += 1;
    if (packed_) {
        if (which == 1)
            SIHG_CUDA(launch_chained(k_step_dual_packed, grid_, kThreads, 0, s, B_, rows_, V_, st,
                                     (const float4*)pack_.as<float4>(), N_));
        else
            SIHG_CUDA(launch_chained(k_step_kty_packed, grid_, kThreads, 0, s, cols_, V_, st, pack_.as<float4>(), N_));
        return SIH_PDHG_OK;
    }
    if (which == 1) {
        if (stage_x_ > 0)
            SIHG_CUDA(launch_chained(k_step_dual_staged, sm_count_, kStagedThreads, sizeof(float) * stage_x_, s, B_,
                                     rows_, V_, st, stage_x_));
        else
            SIHG_CUDA(launch_chained(k_step_dual, grid_, kThreads, 0, s, B_, rows_, V_, st));
    } else {
        if (stage_y_ > 0)
            SIHG_CUDA(launch_chained(k_step_kty_staged, sm_count_, kStagedThreads, sizeof(float) * stage_y_, s,
                                     cols_, V_, st, stage_y_));
        else
            SIHG_CUDA(launch_chained(k_step_kty, grid_, kThreads, 0, s, cols_, V_, st));
    }
    return SIH_PDHG_OK;
}

// Staged gathers (single LP): the first entries of the gathered vector that
// fit in options.staged_kib of shared memory (automatic: the block opt-in
// limit, at most 128 KiB) are staged on a side when, after the renumbering by
// length, their segments on the other side hold at least kStagedShare of the
// nonzeros; the staged kernels run one block per SM.
int MixedSolver::choose_staging() {
    constexpr double kStagedShare = 0.5;
    stage_x_ = stage_y_ = 0;
    if (B_ != 1 || opts_.staged_kib < 0 || nnz_ == 0) return SIH_PDHG_OK;
    int dev = 0, optin = 0;
    SIHG_CUDA(cudaGetDevice(&dev));
    SIHG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    size_t bytes = std::min<size_t>((size_t)optin, 128u * 1024u);
    if (opts_.staged_kib > 0) {
        bytes = (size_t)opts_.staged_kib * 1024u;
        if (bytes > (size_t)optin)
            return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "options.staged_kib exceeds the shared memory of a block");
    }
    const int cap = (int)(bytes / sizeof(float));
    // entries [0, P) of the vector, P a multiple of 4; share of the nonzeros they carry
    auto pick_prefix = [&](const std::vector<int>& ptr, int cnt) -> int {
        const int P = std::min(cap, cnt) & ~3;
        if (P <= 0) return 0;
        const double share = (double)(ptr[P] - ptr[0]) / (double)nnz_;
        return (opts_.staged_kib > 0 || share >= kStagedShare) ? P : 0;
    };
    stage_x_ = pick_prefix(h_csc_ptr_, N_);  // K x' gathers x' by column
    stage_y_ = pick_prefix(h_csr_ptr_, M_);  // K^T y' gathers y' by row
    auto enable = [&](const void* fn, int P, int& out) -> int {
        if (P == 0) return SIH_PDHG_OK;
        const int smem = (int)(sizeof(float) * P);
        SIHG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        int occ = 0;
        SIHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kStagedThreads, smem));
        if (occ < 1) out = 0;
        return SIH_PDHG_OK;
    };
    SIHG_TRY(enable((const void*)k_step_dual_staged, stage_x_, stage_x_));
    SIHG_TRY(enable((const void*)k_step_kty_staged, stage_y_, stage_y_));
    stage_x_rule_ = stage_x_;
    stage_y_rule_ = stage_y_;
    if (opts_.verbose)
        std::fprintf(stderr, "sih_pdhg setup: staged gathers: %d entries of x, %d of y\n", stage_x_, stage_y_);
    return SIH_PDHG_OK;
}

int MixedSolver::launch_eval(cudaStream_t s) {
    launches_ += 4;
    Inst* st = state_.as<Inst>();
    k_flush_avg<<<elem_grid_, kThreads, 0, s>>>(chunks_all_, V_, st);
    k_eval_rows<<<grid_, kThreads, 0, s>>>(rows_, V_, st);
    k_eval_cols<<<grid_, kThreads, 0, s>>>(cols_, V_, st, done_count_.as<unsigned>());
    k_restart<<<elem_grid_, kThreads, 0, s>>>(chunks_all_, V_, st);
    if (packed_ && persistent_ == 0) {  // records of the (possibly restarted) current points
        k_pack<<<elem_grid_, kThreads, 0, s>>>(chunks_all_, V_, st, pack_.as<float4>(), N_);
        launches_ += 1;
    }
    SIHG_LAUNCH_CHECK();
    return launch_compact(s);
}

int MixedSolver::launch_compact(cudaStream_t s) {
    launches_ += 2;
    Inst* st = state_.as<Inst>();
    int* off = layout_.compaction_offsets();
    k_compact_offsets<<<1, 1024, 0, s>>>(B_, st, rows_.inst_task_begin, cols_.inst_task_begin,
                                         chunks_all_.inst_begin, off, rows_.nactive, rows_.counters,
                                         cols_.counters);
    k_compact_fill<<<elem_grid_, kThreads, 0, s>>>(B_, st, rows_, cols_, chunks_all_, off);
    SIHG_LAUNCH_CHECK();
    return SIH_PDHG_OK;
}

int MixedSolver::reset_state() {
    cudaStream_t s = stream_;
    const int g = sm_count_ * 4;
    for (int b = 0; b < B_; ++b) {
        Inst& S = host_inst_[b];
        S.done = 0;
        S.cur = 0;
        S.avg_pending = 0;
        S.restart_flag = 0;
        S.refine = opts_.compensated == 2 ? 1 : 0;
        S.out_sel = 0;
        S.attempts = S.steps = S.rejections = S.restarts = S.since_restart = S.evals = 0;
        S.W = 0.0;
        S.avg_w = 0.0;
        S.kkt_last = S.kkt_prev = 0.0;
        S.tol_p = cfg_.tol_primal;
        S.tol_d = cfg_.tol_dual;
        S.tol_g = cfg_.tol_gap;
        S.verify_rounds = 0;
    }
    SIHG_CUDA(cudaMemcpyAsync(state_.as<Inst>(), host_inst_.data(), sizeof(Inst) * B_, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemsetAsync(done_count_.as<void>(), 0, sizeof(unsigned), s));
    launches_ += 5;
    SIHG_TRY(launch_compact(s));  // every instance runs: full task and chunk lists
    // initial point x = clip(0, l~, u~), y = 0; averages and last points equal it
    k_init_point<<<g, 256, 0, s>>>(N_, M_, V_);
    SIHG_LAUNCH_CHECK();
    bool warm = false;
    for (int b = 0; b < B_; ++b) {
        if (start_x_.size() <= (size_t)b || start_x_[b].empty()) continue;
        warm = true;
        const int co = col_off_[b], ro = row_off_[b], n = probs_[b]->n, m = probs_[b]->m;
        SIHG_CUDA(cudaMemcpyAsync(V_.x1 + co, start_x_[b].data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
        SIHG_CUDA(cudaMemcpyAsync(V_.y1 + ro, start_y_[b].data(), sizeof(float) * m, cudaMemcpyHostToDevice, s));
        k_apply_start<<<std::max(1, std::min(g, (std::max(n, m) + 255) / 256)), 256, 0, s>>>(co, co + n, ro, ro + m, V_);
        launches_ += 1;
    }
    SIHG_LAUNCH_CHECK();
    k_spmv_store<<<grid_, kThreads, 0, s>>>(rows_, state_.as<Inst>(), V_.x0, V_.kx0);
    if (warm) {  // K^T y of the start point (zero for a cold start)
        k_spmv_store<<<grid_, kThreads, 0, s>>>(cols_, state_.as<Inst>(), V_.y0, V_.kty0);
        launches_ += 1;
    }
    k_init_stats_rows<<<grid_, kThreads, 0, s>>>(rows_, V_, state_.as<Inst>());
    k_init_stats_cols<<<grid_, kThreads, 0, s>>>(cols_, V_, state_.as<Inst>());
    k_init_controller<<<(B_ + 127) / 128, 128, 0, s>>>(B_, state_.as<Inst>(), 1.0);
    SIHG_LAUNCH_CHECK();
    // initial evaluation: KKT of the starting point (no restart decision)
    SIHG_TRY(launch_eval(s));
    return SIH_PDHG_OK;
}

int MixedSolver::record_graph() {
    if (graphs_[0]) return SIH_PDHG_OK;
    const unsigned long long saved = launches_;
    cudaGraph_t g = nullptr;
    SIHG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    int rc = SIH_PDHG_OK;
    for (int k = 0; k < eval_freq_ && rc == SIH_PDHG_OK; ++k) rc = launch_step(stream_);
    if (rc == SIH_PDHG_OK) rc = launch_eval(stream_);
    cudaError_t e = cudaStreamEndCapture(stream_, &g);
    if (rc != SIH_PDHG_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    e = cudaGraphInstantiate(&graphs_[0], g, 0);
    cudaGraphDestroy(g);
    launches_ = saved;  // capturing launches nothing
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
    return SIH_PDHG_OK;
}

int MixedSolver::run() {
    eval_freq_ = opts_.eval_frequency > 0 ? opts_.eval_frequency : 64;
    const bool graph = opts_.use_graph && !persistent_;
    if (graph) SIHG_TRY(record_graph());
    if (persistent_) SIHG_CUDA(cudaMemsetAsync(bar_.as<void>(), 0, 4 * sizeof(unsigned), stream_));
    const auto t0 = std::chrono::steady_clock::now();
    launches_ = 0;
    SIHG_TRY(reset_state());
    cudaStream_t s = stream_;
    constexpr int kWindow = 3;
    unsigned* h_done = nullptr;
    SIHG_CUDA(cudaHostAlloc(&h_done, sizeof(unsigned) * kWindow, cudaHostAllocDefault));
    cudaEvent_t ev[kWindow] = {};
    int rc = SIH_PDHG_OK;
    for (int w = 0; w < kWindow && rc == SIH_PDHG_OK; ++w) {
        h_done[w] = 0;
        cudaError_t e = cudaEventCreateWithFlags(&ev[w], cudaEventDisableTiming);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaEventCreate", __FILE__, __LINE__);
    }
    // the evaluation that ends block k sees attempts <= (k + 1) * eval_freq and
    // stops every instance at the iteration limit, so this many blocks suffice
    const long long max_blocks = std::max<long long>(1, (cfg_.max_iterations + eval_freq_ - 1) / eval_freq_);
    long long blk = 0, blk_end = max_blocks;
    timed_out_ = false;
    // Blocks of eval_freq steps and one evaluation until every instance
    // stopped (a window of kWindow blocks in flight; the done count of the
    // oldest is read back before the next is queued).
    auto run_blocks = [&]() -> int {
        for (long long k = 0; blk < blk_end; ++blk, ++k) {
            const int slot = (int)(k % kWindow);
            if (k >= kWindow) {
                cudaError_t e = cudaEventSynchronize(ev[slot]);
                if (e != cudaSuccess) return cuda_fail(e, "cudaEventSynchronize", __FILE__, __LINE__);
                if ((int)h_done[slot] >= B_) break;
                if (opts_.time_limit_sec > 0 &&
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > opts_.time_limit_sec) {
                    timed_out_ = true;
                    break;
                }
            }
            if (persistent_) {
                SIHG_TRY(launch_persistent(s, eval_freq_));
                SIHG_TRY(launch_eval(s));
            } else if (graph) {
                cudaError_t e = cudaGraphLaunch(graphs_[0], s);
                if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch", __FILE__, __LINE__);
                launches_ += (packed_ ? 2ull : 3ull) * eval_freq_ + (packed_ ? 7ull : 6ull);
            } else {
                for (int j = 0; j < eval_freq_; ++j) SIHG_TRY(launch_step(s));
                SIHG_TRY(launch_eval(s));
            }
            cudaMemcpyAsync(&h_done[slot], done_count_.as<unsigned>(), sizeof(unsigned), cudaMemcpyDeviceToHost, s);
            cudaEventRecord(ev[slot], s);
        }
        cudaEventRecord(ev_stop_, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(e, "iteration loop", __FILE__, __LINE__);
        if (persistent_) {
            int status = 0;
            SIHG_CUDA(cudaMemcpy(&status, bar_.as<unsigned long long>() + 1, sizeof(int), cudaMemcpyDeviceToHost));
            if (status != 0)
                return fail(SIH_PDHG_ERR_CUDA, "persistent step kernel: a grid barrier wait ran out (a block stopped "
                                               "arriving); the solve was abandoned");
        }
        SIHG_CUDA(cudaMemcpy(host_inst_.data(), state_.as<Inst>(), sizeof(Inst) * B_, cudaMemcpyDeviceToHost));
        return SIH_PDHG_OK;
    };
    if (rc == SIH_PDHG_OK) {
        cudaEventRecord(ev_start_, s);
        rc = run_blocks();
    }
    // The device stops an instance on relative KKT measures of its FP32 data
    // and iterates (compensated, FP64 totals); the FP64 check of the returned
    // point against the original FP64 problem can read a few percent higher
    // near the tolerance.  An instance whose FP64 check fails goes on with its
    // device tolerances scaled by 0.8 (at most kVerifyRounds times), so that a
    // result reported optimal meets the tolerance in FP64.
    constexpr int kVerifyRounds = 4;
    for (int round = 0; rc == SIH_PDHG_OK && round <= kVerifyRounds && !timed_out_; ++round) {
        std::vector<int> redo;
        std::vector<double> x, y;
        for (int b = 0; b < B_ && rc == SIH_PDHG_OK; ++b) {
            const Inst& S = host_inst_[b];
            if (S.done != 1) continue;
            rc = fetch(b, x, y);
            if (rc != SIH_PDHG_OK) break;
            const KktReport k = host_kkt(probs_[b]->src, x.data(), y.data(), nullptr, nullptr);
            if (!(k.rel_primal <= cfg_.tol_primal && k.rel_dual <= cfg_.tol_dual && k.rel_gap <= cfg_.tol_gap))
                redo.push_back(b);
        }
        if (rc != SIH_PDHG_OK || redo.empty()) break;
        if (round == kVerifyRounds) {  // still above the tolerance in FP64: not reported as optimal
            for (int b : redo) host_inst_[b].done = 4;
            break;
        }
        // blocks enough for the re-opened instance with the fewest attempts to
        // reach the iteration limit (the evaluation stops each at its limit)
        long long min_attempts = cfg_.max_iterations;
        for (int b : redo) min_attempts = std::min(min_attempts, host_inst_[b].attempts);
        blk_end = blk + std::max<long long>(1, (cfg_.max_iterations - min_attempts + eval_freq_ - 1) / eval_freq_);
        for (int b : redo) {
            Inst& S = host_inst_[b];
            S.done = 0;
            S.tol_p *= 0.8;
            S.tol_d *= 0.8;
            S.tol_g *= 0.8;
            S.verify_rounds += 1;
            cudaError_t e = cudaMemcpyAsync(state_.as<Inst>() + b, &S, sizeof(Inst), cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMemcpyAsync", __FILE__, __LINE__); break; }
        }
        if (rc != SIH_PDHG_OK) break;
        unsigned ndone = 0;
        for (int b = 0; b < B_; ++b) ndone += host_inst_[b].done != 0 ? 1u : 0u;
        cudaError_t e = cudaMemcpyAsync(done_count_.as<unsigned>(), &ndone, sizeof(unsigned), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) { rc = cuda_fail(e, "cudaMemcpyAsync", __FILE__, __LINE__); break; }
        for (int w = 0; w < kWindow; ++w) h_done[w] = 0;
        rc = launch_compact(s);  // the re-opened instances' tasks and chunks join the active lists
        if (rc == SIH_PDHG_OK) rc = run_blocks();
    }
    for (int w = 0; w < kWindow; ++w)
        if (ev[w]) cudaEventDestroy(ev[w]);
    cudaFreeHost(h_done);
    if (rc != SIH_PDHG_OK) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev_start_, ev_stop_);
    loop_seconds_ = ms * 1e-3;
    return SIH_PDHG_OK;
}

int MixedSolver::fetch(int b, std::vector<double>& x, std::vector<double>& y) {
    const Inst& S = host_inst_[b];
    const int n = probs_[b]->n, m = probs_[b]->m, co = col_off_[b], ro = row_off_[b];
    std::vector<float> xs(n), ys(m), dc(n), dr(m);
    const float* xsrc = S.out_sel == 1 ? V_.x_avg : (S.cur ? V_.x1 : V_.x0);
    const float* ysrc = S.out_sel == 1 ? V_.y_avg : (S.cur ? V_.y1 : V_.y0);
    SIHG_CUDA(cudaMemcpy(xs.data(), xsrc + co, sizeof(float) * n, cudaMemcpyDeviceToHost));
    SIHG_CUDA(cudaMemcpy(ys.data(), ysrc + ro, sizeof(float) * m, cudaMemcpyDeviceToHost));
    SIHG_CUDA(cudaMemcpy(dc.data(), V_.dcol + co, sizeof(float) * n, cudaMemcpyDeviceToHost));
    SIHG_CUDA(cudaMemcpy(dr.data(), V_.drow + ro, sizeof(float) * m, cudaMemcpyDeviceToHost));
    x.resize(n);
    y.resize(m);
    for (int j = 0; j < n; ++j) x[col_perm_[co + j]] = (double)xs[j] * (double)dc[j];
    for (int i = 0; i < m; ++i) y[row_perm_[ro + i]] = (double)ys[i] * (double)dr[i];
    return SIH_PDHG_OK;
}

// Kernel timing: every instance with a step-weighted average update pending
// (weight 1/2), as after an accepted step.
__global__ void k_mark_average_pending(int B, Inst* __restrict__ st) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        st[b].avg_pending = 1;
        st[b].avg_w = 0.5;
    }
}

int MixedSolver::time_kernels(int reps, double* seconds, double* bytes) {
    SIHG_TRY(reset_state());
    cudaStream_t s = stream_;
    Inst* st = state_.as<Inst>();
    // the state of an accepted step: an average update pending, so that the
    // elementwise pass moves the float-float averages as it does in a solve
    k_mark_average_pending<<<std::max(1, std::min(sm_count_, (B_ + 255) / 256)), 256, 0, s>>>(B_, st);
    SIHG_LAUNCH_CHECK();
    cudaEvent_t e0, e1;
    SIHG_CUDA(cudaEventCreate(&e0));
    SIHG_CUDA(cudaEventCreate(&e1));
    int rc = SIH_PDHG_OK;
    for (int k = 0; k < 3 && rc == SIH_PDHG_OK; ++k) {
        cudaEventRecord(e0, s);
        for (int i = 0; i < reps; ++i) {
            int r = SIH_PDHG_OK;
            if (k == 0) {
                if (packed_) break;  // no elementwise kernel in the packed step
                const cudaError_t e = launch_chained(k_step_primal, elem_grid_, kThreads, 0, s, B_, chunks_all_, V_, st);
                if (e != cudaSuccess) r = cuda_fail(e, "k_step_primal launch", __FILE__, __LINE__);
            } else {
                r = launch_step_spmvs(s, k);
            }
            if (r != SIH_PDHG_OK) {
                rc = r;
                break;
            }
        }
        cudaEventRecord(e1, s);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) rc = cuda_fail(e, "kernel timing", __FILE__, __LINE__);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        seconds[k] = (k == 0 && packed_) ? 0.0 : ms * 1e-3 / reps;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (bytes) {
        // algorithmic bytes of one launch: every array the kernel must touch, once
        const double nnz = (double)nnz_, m = M_, n = N_;
        if (packed_) {
            bytes[0] = 0.0;
            // pairs, ptr, a 16-byte record per column gathered, row epilogue with the y average
            bytes[1] = 8.0 * nnz + 4.0 * (m + 1) + 16.0 * n + 44.0 * m;
            // pairs, ptr, y' gathered; per column: record, K^T y, c in; x', K^T y', record out; x average in+out
            bytes[2] = 8.0 * nnz + 4.0 * (n + 1) + 4.0 * m + 60.0 * n;
        } else {
            bytes[0] = 40.0 * n + 20.0 * m;                   // x,K^T y,c,l,u in, x' out, x/y averages in+out
            bytes[1] = 8.0 * nnz + 4.0 * (m + 1) + 4.0 * n + 28.0 * m;  // pairs, ptr, x' gathered, row epilogue
            bytes[2] = 8.0 * nnz + 4.0 * (n + 1) + 4.0 * m + 16.0 * n;  // pairs, ptr, y' gathered, column epilogue
        }
    }
    return rc;
}

// Start point for instance b from the next run on: x (original column order)
// and y (original row order, in the convention of the returned row_duals,
// options.dual_sign); omega > 0 also sets the initial primal weight.  NULL x
// clears the start.
int MixedSolver::set_start(int b, const double* x, const double* y, double omega) {
    if (b < 0 || b >= B_) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "instance index out of range");
    start_x_.resize(B_);
    start_y_.resize(B_);
    if (!x) {
        start_x_[b].clear();
        start_y_[b].clear();
        host_inst_[b].omega_start = 0.0;
        return SIH_PDHG_OK;
    }
    const int n = probs_[b]->n, m = probs_[b]->m, co = col_off_[b], ro = row_off_[b];
    start_x_[b].assign(n, 0.f);
    start_y_[b].assign(m, 0.f);
    for (int j = 0; j < n; ++j) {
        const double v = x[col_perm_[co + j]];
        if (!std::isfinite(v)) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "start x is not finite");
        start_x_[b][j] = (float)v;
    }
    for (int i = 0; i < m; ++i) {
        const double v = y ? y[row_perm_[ro + i]] : 0.0;
        if (!std::isfinite(v)) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "start y is not finite");
        // same convention as the returned row_duals (options.dual_sign)
        start_y_[b][i] = (float)(opts_.dual_sign ? -v * probs_[b]->sense : v);
    }
    host_inst_[b].omega_start = omega > 0.0 && std::isfinite(omega) ? omega : 0.0;
    return SIH_PDHG_OK;
}

// Launch-shape autotuner (options.autotune): on this batch, times the two
// step SpMVs over
//   * the nonzeros per task (a ladder around the default),
//   * the lanes per segment of the light tasks of each side (the length rule,
//     or 1, 2, 4, 8 forced),
//   * the staged gathers of a single LP (on / off per side),
// one coordinate after the other, keeping the fastest, then (options.persistent
// < 0) the step form: kernels per phase replayed as a graph, or the persistent
// kernel, by the device time of a block of steps and an evaluation.  The
// choice is cached per process for the shape (instances, rows, columns,
// nonzeros), so repeated solves of one shape tune once.
namespace {
struct TuneKey {
    int b, m, n;
    long long nnz;
    bool operator<(const TuneKey& o) const { return std::tie(b, m, n, nnz) < std::tie(o.b, o.m, o.n, o.nnz); }
};
std::mutex g_tune_mu;
std::map<TuneKey, sih_pdhg_launch_shape> g_tune_cache;
}  // namespace

void MixedSolver::launch_shape(sih_pdhg_launch_shape* out) const {
    out->task_nnz = task_nnz_;
    out->row_lanes = lanes_r_;
    out->col_lanes = lanes_c_;
    out->staged_x = stage_x_;
    out->staged_y = stage_y_;
    out->persistent = persistent_;
    out->grid = persistent_ ? pgrid_ : grid_;
    out->tuned = tuned_;
    out->packed = packed_;
    out->reserved = 0;
}

// A cached shape; what the caller's options fix stays as they say.
int MixedSolver::apply_shape(const sih_pdhg_launch_shape& sh) {
    if (opts_.lanes_csr == 0) lanes_r_ = sh.row_lanes;
    if (opts_.lanes_csc == 0) lanes_c_ = sh.col_lanes;
    SIHG_TRY(build_schedules(opts_.tile_nnz > 0 ? task_nnz_ : sh.task_nnz));
    stage_x_ = sh.staged_x ? stage_x_rule_ : 0;
    stage_y_ = sh.staged_y ? stage_y_rule_ : 0;
    return opts_.persistent < 0 ? set_form(sh.persistent) : SIH_PDHG_OK;
}

// Device seconds of one block of eval_freq steps and an evaluation in the
// current step form, from the initial point (after one untimed block).
int MixedSolver::time_block(double* seconds) {
    eval_freq_ = opts_.eval_frequency > 0 ? opts_.eval_frequency : 64;
    const bool graph = opts_.use_graph && !persistent_;
    if (graph) SIHG_TRY(record_graph());
    if (persistent_) SIHG_CUDA(cudaMemsetAsync(bar_.as<void>(), 0, 4 * sizeof(unsigned), stream_));
    SIHG_TRY(reset_state());
    cudaStream_t s = stream_;
    auto block = [&]() -> int {
        if (persistent_) {
            SIHG_TRY(launch_persistent(s, eval_freq_));
            return launch_eval(s);
        }
        if (graph) {
            SIHG_CUDA(cudaGraphLaunch(graphs_[0], s));
            return SIH_PDHG_OK;
        }
        for (int j = 0; j < eval_freq_; ++j) SIHG_TRY(launch_step(s));
        return launch_eval(s);
    };
    SIHG_TRY(block());
    constexpr int kBlocks = 2;
    SIHG_CUDA(cudaEventRecord(ev_start_, s));
    for (int k = 0; k < kBlocks; ++k) SIHG_TRY(block());
    SIHG_CUDA(cudaEventRecord(ev_stop_, s));
    SIHG_CUDA(cudaEventSynchronize(ev_stop_));
    float ms = 0.f;
    SIHG_CUDA(cudaEventElapsedTime(&ms, ev_start_, ev_stop_));
    *seconds = ms * 1e-3 / kBlocks;
    return SIH_PDHG_OK;
}

int MixedSolver::autotune() {
    const TuneKey key{B_, M_, N_, nnz_};
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            SIHG_TRY(apply_shape(it->second));
            tuned_ = 1;
            return SIH_PDHG_OK;
        }
    }
    const int reps = nnz_ > 64000000 ? 3 : (nnz_ > 4000000 ? 5 : 20);
    double sec[3];
    auto time_sides = [&](double& rows_s, double& cols_s) -> int {
        SIHG_TRY(time_kernels(reps, sec, nullptr));
        rows_s = sec[1];
        cols_s = sec[2];
        return SIH_PDHG_OK;
    };
    // A candidate replaces the incumbent (the rule's choice first) only when it
    // is faster by more than kTuneMargin: timing noise then does not flip the
    // shape from one process to the next (the shape sets the summation order,
    // so it also decides the exact trajectory of the iterates).
    constexpr double kTuneMargin = 0.97;
    double tr = 0, tc = 0;
    // task size (lanes as configured)
    int best_t = task_nnz_;
    if (opts_.tile_nnz <= 0) {
        std::vector<int> ladder = {384, 768, 1536};
        if (nnz_ <= 64000000) ladder.insert(ladder.end(), {256, 512, 1024, 2048});
        std::sort(ladder.begin(), ladder.end());
        ladder.erase(std::unique(ladder.begin(), ladder.end()), ladder.end());
        ladder.insert(ladder.begin(), task_nnz_);  // the incumbent, timed first
        double best = INFINITY;
        for (size_t k = 0; k < ladder.size(); ++k) {
            const int t = ladder[k];
            if (k > 0 && t == task_nnz_) continue;
            if ((long long)t > std::max<long long>(nnz_, 256)) continue;
            SIHG_TRY(build_schedules(t));
            SIHG_TRY(time_sides(tr, tc));
            if (k == 0 || tr + tc < kTuneMargin * best) {
                best = tr + tc;
                best_t = t;
            }
        }
    }
    // lanes per segment of each side's light tasks (0 = the length rule)
    const std::vector<int> lane_ladder = {0, 1, 2, 4, 8};
    for (int side = 0; side < 2; ++side) {
        if ((side == 0 ? opts_.lanes_csr : opts_.lanes_csc) != 0) continue;  // fixed by the caller
        int& lanes = side == 0 ? lanes_r_ : lanes_c_;
        int best_l = lanes;
        double best = INFINITY;
        for (int L : lane_ladder) {  // the rule (0) first: the incumbent
            lanes = L;
            SIHG_TRY(build_schedules(best_t));
            SIHG_TRY(time_sides(tr, tc));
            const double t = side == 0 ? tr : tc;
            if (L == lane_ladder[0] || t < kTuneMargin * best) {
                best = t;
                best_l = L;
            }
        }
        lanes = best_l;
    }
    SIHG_TRY(build_schedules(best_t));
    // staged gathers (single LP): keep each side's only if it is faster
    for (int side = 0; side < 2; ++side) {
        int& st = side == 0 ? stage_x_ : stage_y_;
        const int rule = side == 0 ? stage_x_rule_ : stage_y_rule_;
        if (rule == 0) continue;
        st = rule;
        SIHG_TRY(time_sides(tr, tc));
        const double on = side == 0 ? tr : tc;
        st = 0;
        SIHG_TRY(time_sides(tr, tc));
        const double off = side == 0 ? tr : tc;
        st = off < kTuneMargin * on ? 0 : rule;
    }
    // step form: graph of kernels per phase, or the persistent kernel
    if (opts_.persistent < 0) {
        const int alt = B_ == 1 ? 2 : 1;
        if ((alt == 1 ? grid_form1_ : grid_form2_) > 0) {
            const int incumbent = persistent_;  // the automatic rule's form
            const int other = incumbent == 0 ? alt : 0;
            double t0 = 0, t1 = 0;
            SIHG_TRY(time_block(&t0));
            SIHG_TRY(set_form(other));
            SIHG_TRY(time_block(&t1));
            SIHG_TRY(set_form(t1 < kTuneMargin * t0 ? other : incumbent));
        }
    }
    tuned_ = 1;
    sih_pdhg_launch_shape sh{};
    launch_shape(&sh);
    if (opts_.verbose)
        std::fprintf(stderr, "sih_pdhg autotune: task_nnz %d, lanes rows %d cols %d, staged %d/%d, form %d\n",
                     sh.task_nnz, sh.row_lanes, sh.col_lanes, sh.staged_x, sh.staged_y, sh.persistent);
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache[key] = sh;
    return SIH_PDHG_OK;
}

int solve_mixed(const HostProblem& hp, const sih_pdhg_config& cfg, const sih_pdhg_options& opts,
                sih_pdhg_result* r) {
    using clk = std::chrono::steady_clock;
    auto secs = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); };
    const auto t0 = clk::now();
    MixedSolver solver;
    std::vector<const HostProblem*> probs{&hp};
    SIHG_TRY(solver.setup(probs, cfg, opts));
    cudaStreamSynchronize(solver.stream());
    const auto t1 = clk::now();
    SIHG_TRY(solver.run());
    const auto t2 = clk::now();
    std::vector<double> x, y;
    SIHG_TRY(solver.fetch(0, x, y));
    const auto t3 = clk::now();
    solver.fill_result(0, r);
    pack_solution(hp.src, opts, x, y, r);
    if (opts.verbose)
        std::fprintf(stderr, "sih_pdhg mixed: setup %.3f s, run %.3f s (device %.3f s), fetch %.3f s, pack %.3f s\n",
                     secs(t0, t1), secs(t1, t2), solver.loop_seconds(), secs(t2, t3), secs(t3, clk::now()));
    r->d2h_bytes = 8ull * (hp.n + hp.m);
    r->h2d_bytes = mixed_h2d_bytes(hp);
    return SIH_PDHG_OK;
}

void MixedSolver::fill_result(int b, sih_pdhg_result* r) const {
    const Inst& S = host_inst_[b];
    switch (S.done) {
        case 1: r->status = SIH_STATUS_OPTIMAL; break;
        case 2: r->status = SIH_STATUS_ITERATION_LIMIT; break;
        case 3: r->status = SIH_STATUS_NUMERICAL_FAILURE; break;
        // the device test passed, the FP64 check of the point failed after the
        // verification rounds: the FP32 data cannot get this instance closer
        case 4: r->status = SIH_STATUS_NUMERICAL_FAILURE; break;
        default: r->status = timed_out_ ? SIH_STATUS_TIME_LIMIT : SIH_STATUS_ITERATION_LIMIT; break;
    }
    r->iterations = S.attempts;
    r->restarts = S.restarts;
    r->step_rejections = S.rejections;
    r->final_step = S.eta;
    r->final_primal_weight = S.omega;
    r->ref_primal = S.rel_p[S.out_sel];
    r->ref_dual = S.rel_d[S.out_sel];
    r->time_solver_sec = loop_seconds_;
    r->kernel_launches = launches_;
}

}  // namespace sihg
