// Plain FP32 PDHG with the reference's semantics, as sm_103a kernels.
//
// Per iteration (core/src/gpu/gpu_solver.cpp:227-239) the reference launches
// four kernels: CSC SpMV A^T y, the primal update, CSR SpMV A x_bar and the dual
// update.  Here the SpMVs and their updates are fused:
//   plain_primal_kernel : z_j = (A^T y)_j (CSC)  ->  x, x_bar update   (cuda_pdhg.cu:33-77)
//   plain_dual_kernel   : w_i = (A x_bar)_i (CSR) ->  y update         (cuda_pdhg.cu:14-30, 82-103)
// so A^T y and A x_bar never reach HBM.  The reference's restart kernel
// (x_bar <- x every 250 iterations, cuda_pdhg.cu:106-111) has no effect on the
// iterates because the next primal update overwrites x_bar before it is read,
// so it is not launched.
//
// Every check_frequency iterations (and at max_iterations) the reference
// recomputes A x and A^T y, copies the per-row / per-column violation maps to
// the host and takes their maxima there (gpu_solver.cpp:242-269).  Here the
// violations are reduced on the device (exact float max), a one-thread kernel
// applies the reference's tests, and the best iterate is copied on the device;
// the host only polls a done flag.  The iteration blocks between checks are
// replayed as CUDA graphs.
#include <algorithm>
#include <chrono>

#include "plain.h"
#include "spmv.cuh"
#include "warp.cuh"

namespace sihg {

// ---------------------------------------------------------------- kernels
// Primal update of column j with z = (A^T y)_j (cuda_pdhg.cu:54-77).
struct PrimalEpi {
    PlainVecs v;
    struct Pre { float x, c, tau, l, u; };
    __device__ __forceinline__ Pre pre(int j) const { return Pre{v.x[j], v.c[j], v.tau[j], v.l[j], v.u[j]}; }
    __device__ __forceinline__ void apply(int j, float aty, const Pre& p) const {
        const float grad = __fadd_rn(p.c, aty);
        float x_new = __fsub_rn(p.x, __fmul_rn(p.tau, grad));
        if (x_new < p.l) x_new = p.l;
        if (x_new > p.u) x_new = p.u;
        v.x[j] = x_new;
        v.xbar[j] = __fsub_rn(__fmul_rn(2.0f, x_new), p.x);
    }
};

// Dual update of row i with w = (A x_bar)_i (cuda_pdhg.cu:82-103).
struct DualEpi {
    PlainVecs v;
    struct Pre { float sig, y, rl, ru; };
    __device__ __forceinline__ Pre pre(int i) const { return Pre{v.sigma[i], v.y[i], v.rl[i], v.ru[i]}; }
    __device__ __forceinline__ void apply(int i, float axbar, const Pre& p) const {
        const float w = __fadd_rn(axbar, p.y / p.sig);
        float q = w;
        if (q < p.rl) q = p.rl;
        if (q > p.ru) q = p.ru;
        v.y[i] = __fmul_rn(p.sig, __fsub_rn(w, q));
    }
};

// Row violation of A x (cuda_pdhg.cu:114-129), running max per thread.
struct RowViolEpi {
    PlainVecs v;
    float lmax;
    struct Pre { float rl, ru; };
    __device__ __forceinline__ Pre pre(int i) const { return Pre{v.rl[i], v.ru[i]}; }
    __device__ __forceinline__ void apply(int, float ax, const Pre& p) {
        float viol = 0.0f;
        if (p.rl > -1e15f && ax < p.rl) viol = fmaxf(viol, __fsub_rn(p.rl, ax));
        if (p.ru < 1e15f && ax > p.ru) viol = fmaxf(viol, __fsub_rn(ax, p.ru));
        lmax = fmaxf(lmax, viol);
    }
};

// Column measure |x - clip(x - tau (c + A^T y))| / max(1e-4, tau) (cuda_pdhg.cu:131-151).
// fmaxf drops NaN measures, as the reference's host std::max does.
struct ColMeasEpi {
    PlainVecs v;
    float lmax;
    struct Pre { float x, c, tau, l, u; };
    __device__ __forceinline__ Pre pre(int j) const { return Pre{v.x[j], v.c[j], v.tau[j], v.l[j], v.u[j]}; }
    __device__ __forceinline__ void apply(int, float aty, const Pre& p) {
        float proj = __fsub_rn(p.x, __fmul_rn(p.tau, __fadd_rn(p.c, aty)));
        if (proj < p.l) proj = p.l;
        if (proj > p.u) proj = p.u;
        lmax = fmaxf(lmax, fabsf(__fsub_rn(p.x, proj)) / fmaxf(1e-4f, p.tau));
    }
};

template <bool EXACT>
__global__ void __launch_bounds__(256, 8) plain_primal_kernel(SegMatrix At, SpmvPlan P, PlainVecs v,
                                                           const PlainState* __restrict__ st) {
    if (st->done) return;
    PrimalEpi epi{v};
    spmv_run<EXACT>(At, P, v.y, epi);
}

template <bool EXACT>
__global__ void __launch_bounds__(256, 8) plain_dual_kernel(SegMatrix A, SpmvPlan P, PlainVecs v,
                                                         const PlainState* __restrict__ st) {
    if (st->done) return;
    DualEpi epi{v};
    spmv_run<EXACT>(A, P, v.xbar, epi);
}

// Fast path of the iteration (exact_arithmetic = 0): the same epilogues on
// the task engine (warp.cuh: dynamic warp tasks, software-pipelined loads).
template <class E>
struct PlainTaskEpi {
    E e;
    const float* vec;
    using Pre = typename E::Pre;
    __device__ __forceinline__ Pre pre(int k) const { return e.pre(k); }
    __device__ __forceinline__ void begin(const PlainState&) {}
    __device__ __forceinline__ const float* gather(int) const { return vec; }
    __device__ __forceinline__ void apply(int k, const SegDot<1>& d, const Pre& p) { e.apply(k, d.s[0], p); }
};

__global__ void __launch_bounds__(kThreads, 4) plain_primal_tasks(Side cols, PlainVecs v, PlainState* st) {
    if (st->done) return;
    PlainTaskEpi<PrimalEpi> epi{PrimalEpi{v}, v.y};
    spmv_engine<1, false, 0>(cols, st, epi, 0u);
}

__global__ void __launch_bounds__(kThreads, 4) plain_dual_tasks(Side rows, PlainVecs v, PlainState* st) {
    if (st->done) return;
    PlainTaskEpi<DualEpi> epi{DualEpi{v}, v.xbar};
    spmv_engine<1, false, 0>(rows, st, epi, 0u);
}

template <bool EXACT>
__global__ void __launch_bounds__(256, 8) plain_check_rows_kernel(SegMatrix A, SpmvPlan P, PlainVecs v,
                                                               PlainState* st) {
    if (st->done) return;
    __shared__ float red[32];
    RowViolEpi epi{v, 0.f};
    spmv_run<EXACT>(A, P, v.x, epi);
    const float b = block_max_nonneg(epi.lmax, red);
    if (threadIdx.x == 0 && b > 0.f) atomicMax(&st->max_p_bits, __float_as_uint(b));
}

template <bool EXACT>
__global__ void __launch_bounds__(256, 8) plain_check_cols_kernel(SegMatrix At, SpmvPlan P, PlainVecs v,
                                                               PlainState* st) {
    if (st->done) return;
    __shared__ float red[32];
    ColMeasEpi epi{v, 0.f};
    spmv_run<EXACT>(At, P, v.y, epi);
    const float b = block_max_nonneg(epi.lmax, red);
    if (threadIdx.x == 0 && b > 0.f) atomicMax(&st->max_d_bits, __float_as_uint(b));
}

// The host part of the reference check (gpu_solver.cpp:252-268), one thread.
__global__ void plain_check_finish_kernel(PlainState* st) {
    if (st->done) {
        st->copy_best = 0;
        return;
    }
    const float max_p = __uint_as_float(st->max_p_bits), max_d = __uint_as_float(st->max_d_bits);
    st->max_p_bits = 0u;
    st->max_d_bits = 0u;
    const float np = max_p / st->max_abs_b, nd = max_d / st->max_abs_c;
    const float comb = (np < nd) ? nd : np;
    const int it = min(st->next_check, st->max_iterations);
    st->next_check += st->check_frequency;
    st->checks += 1;
    st->last_norm_p = np;
    st->last_norm_d = nd;
    st->copy_best = 0;
    if (comb < st->best_combined) {
        st->best_combined = comb;
        st->copy_best = 1;
    }
    if (np <= st->tol_p && nd <= st->tol_d) {
        st->done = 1;
        st->iterations = it;
    }
}

__global__ void plain_copy_best_kernel(int n, const float* __restrict__ x, float* __restrict__ best,
                                       const PlainState* __restrict__ st) {
    if (!st->copy_best) return;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) best[j] = x[j];
}

// Step sizes of gpu_solver.cpp:128-151: 0.95 / max(1, sum |a|) per segment,
// summed in entry order in float, or the configured constant.
__global__ void abs_sum_step_kernel(int nseg, const int* __restrict__ ptr, const int2* __restrict__ pairs,
                                    float fixed, float* __restrict__ out) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += gridDim.x * blockDim.x) {
        float sum = 0.0f;
        for (int k = ptr[s]; k < ptr[s + 1]; ++k) sum = __fadd_rn(sum, fabsf(__int_as_float(pairs[k].y)));
        out[s] = fixed > 0.0f ? fixed : 0.95f / ((1.0f < sum) ? sum : 1.0f);
    }
}

// ---------------------------------------------------------------- host driver
int PlainSolver::setup(const HostProblem& hp, const sih_pdhg_config& cfg, const sih_pdhg_options& opts) {
    hp_ = &hp;
    cfg_ = cfg;
    opts_ = opts;
    exact_ = opts.exact_arithmetic != 0;
    const int m = hp.m, n = hp.n, nnz = hp.nnz;
    int dev = 0;
    SIHG_CUDA(cudaGetDevice(&dev));
    SIHG_CUDA(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, dev));
    SIHG_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    SIHG_CUDA(cudaEventCreate(&ev_start_));
    SIHG_CUDA(cudaEventCreate(&ev_stop_));

    SIHG_TRY(csc_ptr_.alloc(sizeof(int) * (n + 1)));
    SIHG_TRY(csr_ptr_.alloc(sizeof(int) * (m + 1)));
    SIHG_TRY(csc_pairs_.alloc(sizeof(Pair) * nnz));
    SIHG_TRY(csr_pairs_.alloc(sizeof(Pair) * nnz));
    SIHG_TRY(colvec_.alloc(sizeof(float) * (size_t)n * 8));
    SIHG_TRY(rowvec_.alloc(sizeof(float) * (size_t)m * 4));
    SIHG_TRY(state_.alloc(sizeof(PlainState)));

    cudaStream_t s = stream_;
    SIHG_CUDA(cudaMemcpyAsync(csc_ptr_.as<int>(), hp.csc_ptr.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(csr_ptr_.as<int>(), hp.csr_ptr.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice, s));
    if (nnz > 0) {
        SIHG_CUDA(cudaMemcpyAsync(csc_pairs_.as<Pair>(), hp.csc.data(), sizeof(Pair) * nnz, cudaMemcpyHostToDevice, s));
        SIHG_CUDA(cudaMemcpyAsync(csr_pairs_.as<Pair>(), hp.csr.data(), sizeof(Pair) * nnz, cudaMemcpyHostToDevice, s));
    }
    float* cv = colvec_.as<float>();
    float* rv = rowvec_.as<float>();
    // column vectors: c l u tau x xbar best_x (7 used of 8 slots)
    vec_.c = cv + 0 * (size_t)n;
    vec_.l = cv + 1 * (size_t)n;
    vec_.u = cv + 2 * (size_t)n;
    vec_.tau = cv + 3 * (size_t)n;
    vec_.x = cv + 4 * (size_t)n;
    vec_.xbar = cv + 5 * (size_t)n;
    vec_.best_x = cv + 6 * (size_t)n;
    vec_.rl = rv + 0 * (size_t)m;
    vec_.ru = rv + 1 * (size_t)m;
    vec_.sigma = rv + 2 * (size_t)m;
    vec_.y = rv + 3 * (size_t)m;
    SIHG_CUDA(cudaMemcpyAsync(cv + 0 * (size_t)n, hp.c.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(cv + 1 * (size_t)n, hp.l.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(cv + 2 * (size_t)n, hp.u.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(rv + 0 * (size_t)m, hp.rl.data(), sizeof(float) * m, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(rv + 1 * (size_t)m, hp.ru.data(), sizeof(float) * m, cudaMemcpyHostToDevice, s));

    // plans and heavy lists
    std::vector<int> heavy_c, heavy_r;
    plan_csc_ = make_plan(hp.csc_ptr, opts.lanes_csc, opts.heavy_factor, exact_, sm_count_, heavy_c);
    plan_csr_ = make_plan(hp.csr_ptr, opts.lanes_csr, opts.heavy_factor, exact_, sm_count_, heavy_r);
    SIHG_TRY(heavy_.alloc(sizeof(int) * (heavy_c.size() + heavy_r.size() + 1)));
    if (!heavy_c.empty())
        SIHG_CUDA(cudaMemcpyAsync(heavy_.as<int>(), heavy_c.data(), sizeof(int) * heavy_c.size(), cudaMemcpyHostToDevice, s));
    if (!heavy_r.empty())
        SIHG_CUDA(cudaMemcpyAsync(heavy_.as<int>() + heavy_c.size(), heavy_r.data(), sizeof(int) * heavy_r.size(),
                                  cudaMemcpyHostToDevice, s));
    plan_csc_.heavy_idx = heavy_.as<int>();
    plan_csr_.heavy_idx = heavy_.as<int>() + heavy_c.size();
    At_ = SegMatrix{n, csc_ptr_.as<int>(), csc_pairs_.as<int2>()};
    A_ = SegMatrix{m, csr_ptr_.as<int>(), csr_pairs_.as<int2>()};
    if (!exact_ && m > 0 && n > 0) {  // task engine of the fast iteration kernels
        int occ = 0;
        SIHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, plain_primal_tasks, kThreads, 0));
        task_grid_ = sm_count_ * std::max(1, occ);
        const long long warps = (long long)task_grid_ * (kThreads / 32);
        const int task_nnz = opts.tile_nnz > 0
                                 ? opts.tile_nnz
                                 : (int)std::max(128LL, std::min(2048LL, (long long)nnz / std::max(1LL, 3 * warps)));
        SIHG_TRY(layout_.build(hp.csr_ptr, hp.csc_ptr, std::vector<int>{0, m}, std::vector<int>{0, n}, A_, At_,
                               task_nnz, true, s));
    }

    // step sizes on the device, in the reference's summation order
    if (n > 0) {
        abs_sum_step_kernel<<<std::min((n + 255) / 256, sm_count_ * 8), 256, 0, s>>>(
            n, At_.ptr, At_.pairs, cfg.step_tau, cv + 3 * (size_t)n);
        SIHG_LAUNCH_CHECK();
    }
    if (m > 0) {
        abs_sum_step_kernel<<<std::min((m + 255) / 256, sm_count_ * 8), 256, 0, s>>>(
            m, A_.ptr, A_.pairs, cfg.step_sigma, rv + 2 * (size_t)m);
        SIHG_LAUNCH_CHECK();
    }
    // initial point x = clip(0, l, u) (gpu_solver.cpp:192-196), x_bar = x, y = 0
    x0_.resize(n);
    for (int j = 0; j < n; ++j) {
        const float up0 = (0.0f < hp.u[j]) ? 0.0f : hp.u[j];   // std::min(u, 0)
        x0_[j] = (hp.l[j] < up0) ? up0 : hp.l[j];              // std::max(l, .)
    }
    // max |c| and max |b| over finite bounds (gpu_solver.cpp:112-126)
    max_abs_c_ = 1.0f;
    for (int j = 0; j < n; ++j) max_abs_c_ = (max_abs_c_ < std::fabs(hp.c[j])) ? std::fabs(hp.c[j]) : max_abs_c_;
    max_abs_b_ = 1.0f;
    for (int i = 0; i < m; ++i) {
        if (hp.ru[i] < 1e15f) max_abs_b_ = (max_abs_b_ < std::fabs(hp.ru[i])) ? std::fabs(hp.ru[i]) : max_abs_b_;
        if (hp.rl[i] > -1e15f) max_abs_b_ = (max_abs_b_ < std::fabs(hp.rl[i])) ? std::fabs(hp.rl[i]) : max_abs_b_;
    }
    SIHG_TRY(record_graphs());
    return SIH_PDHG_OK;
}

int PlainSolver::launch_iteration(cudaStream_t s) {
    const PlainState* st = state_.as<PlainState>();
    if (exact_) {
        plain_primal_kernel<true><<<plan_csc_.grid(), plan_csc_.threads, 0, s>>>(At_, plan_csc_, vec_, st);
        plain_dual_kernel<true><<<plan_csr_.grid(), plan_csr_.threads, 0, s>>>(A_, plan_csr_, vec_, st);
    } else {
        PlainState* sw = state_.as<PlainState>();
        plain_primal_tasks<<<task_grid_, kThreads, 0, s>>>(layout_.cols, vec_, sw);
        plain_dual_tasks<<<task_grid_, kThreads, 0, s>>>(layout_.rows, vec_, sw);
    }
    SIHG_LAUNCH_CHECK();
    return SIH_PDHG_OK;
}

int PlainSolver::launch_check(cudaStream_t s) {
    PlainState* st = state_.as<PlainState>();
    if (exact_) {
        plain_check_rows_kernel<true><<<plan_csr_.grid(), plan_csr_.threads, 0, s>>>(A_, plan_csr_, vec_, st);
        plain_check_cols_kernel<true><<<plan_csc_.grid(), plan_csc_.threads, 0, s>>>(At_, plan_csc_, vec_, st);
    } else {
        plain_check_rows_kernel<false><<<plan_csr_.grid(), plan_csr_.threads, 0, s>>>(A_, plan_csr_, vec_, st);
        plain_check_cols_kernel<false><<<plan_csc_.grid(), plan_csc_.threads, 0, s>>>(At_, plan_csc_, vec_, st);
    }
    plain_check_finish_kernel<<<1, 1, 0, s>>>(st);
    const int n = hp_->n;
    plain_copy_best_kernel<<<std::max(1, std::min((n + 255) / 256, sm_count_ * 4)), 256, 0, s>>>(n, vec_.x, vec_.best_x, st);
    SIHG_LAUNCH_CHECK();
    return SIH_PDHG_OK;
}

int PlainSolver::record_block(int iters, cudaGraphExec_t* exec) {
    cudaGraph_t g = nullptr;
    SIHG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    int rc = SIH_PDHG_OK;
    if (!exact_ && layout_.rows.counters) {  // the task counters restart with every block
        cudaError_t e = cudaMemsetAsync(layout_.rows.counters, 0, sizeof(unsigned), stream_);
        if (e == cudaSuccess) e = cudaMemsetAsync(layout_.cols.counters, 0, sizeof(unsigned), stream_);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemsetAsync", __FILE__, __LINE__);
    }
    for (int k = 0; k < iters && rc == SIH_PDHG_OK; ++k) rc = launch_iteration(stream_);
    if (rc == SIH_PDHG_OK) rc = launch_check(stream_);
    cudaError_t e = cudaStreamEndCapture(stream_, &g);
    if (rc != SIH_PDHG_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
    return SIH_PDHG_OK;
}

int PlainSolver::record_graphs() {
    if (!opts_.use_graph) return SIH_PDHG_OK;
    const int cf = cfg_.check_frequency;
    const int maxit = cfg_.max_iterations;
    if (maxit >= cf) SIHG_TRY(record_block(cf, &block_exec_));
    if (maxit % cf) SIHG_TRY(record_block(maxit % cf, &tail_exec_));
    return SIH_PDHG_OK;
}

int PlainSolver::reset_state() {
    const int n = hp_->n, m = hp_->m;
    cudaStream_t s = stream_;
    SIHG_CUDA(cudaMemcpyAsync(vec_.x, x0_.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(vec_.xbar, x0_.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(vec_.best_x, x0_.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemsetAsync(vec_.y, 0, sizeof(float) * m, s));
    PlainState st{};
    st.next_check = cfg_.check_frequency;
    st.best_combined = 1e30f;
    st.max_abs_b = max_abs_b_;
    st.max_abs_c = max_abs_c_;
    st.tol_p = cfg_.tol_primal;
    st.tol_d = cfg_.tol_dual;
    st.check_frequency = cfg_.check_frequency;
    st.max_iterations = cfg_.max_iterations;
    host_state_ = st;
    SIHG_CUDA(cudaMemcpyAsync(state_.as<PlainState>(), &host_state_, sizeof(PlainState), cudaMemcpyHostToDevice, s));
    if (!exact_ && layout_.rows.counters) {
        SIHG_CUDA(cudaMemsetAsync(layout_.rows.counters, 0, sizeof(unsigned), s));
        SIHG_CUDA(cudaMemsetAsync(layout_.cols.counters, 0, sizeof(unsigned), s));
    }
    return SIH_PDHG_OK;
}

int PlainSolver::iterate() {
    SIHG_TRY(reset_state());
    const int cf = cfg_.check_frequency;
    const int maxit = cfg_.max_iterations;
    const int nblocks = maxit / cf;
    const int tail = maxit % cf;
    // Poll the done flag through a ring of pinned slots: at most kWindow blocks
    // are in flight past the one that converged, and those exit at once.
    constexpr int kWindow = 4;
    int* h_done = nullptr;
    SIHG_CUDA(cudaHostAlloc(&h_done, sizeof(int) * kWindow, cudaHostAllocDefault));
    cudaEvent_t ev[kWindow] = {};
    int rc = SIH_PDHG_OK;
    for (int w = 0; w < kWindow && rc == SIH_PDHG_OK; ++w) {
        h_done[w] = 0;
        cudaError_t e = cudaEventCreateWithFlags(&ev[w], cudaEventDisableTiming);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaEventCreate", __FILE__, __LINE__);
    }
    launches_ = 0;
    if (rc == SIH_PDHG_OK) {
        cudaStream_t s = stream_;
        cudaEventRecord(ev_start_, s);
        bool done = false;
        for (int b = 0; b < nblocks + (tail ? 1 : 0) && !done && rc == SIH_PDHG_OK; ++b) {
            const int slot = b % kWindow;
            if (b >= kWindow) {
                cudaError_t e = cudaEventSynchronize(ev[slot]);
                if (e != cudaSuccess) { rc = cuda_fail(e, "cudaEventSynchronize", __FILE__, __LINE__); break; }
                if (h_done[slot]) { done = true; break; }
            }
            const bool is_tail = b == nblocks;
            launches_ += 2ull * (is_tail ? tail : cf) + 4ull;
            if (opts_.use_graph) {
                cudaError_t e = cudaGraphLaunch(is_tail ? tail_exec_ : block_exec_, s);
                if (e != cudaSuccess) { rc = cuda_fail(e, "cudaGraphLaunch", __FILE__, __LINE__); break; }
            } else {
                const int its = is_tail ? tail : cf;
                if (!exact_ && layout_.rows.counters) {  // task counters restart with every block
                    cudaMemsetAsync(layout_.rows.counters, 0, sizeof(unsigned), s);
                    cudaMemsetAsync(layout_.cols.counters, 0, sizeof(unsigned), s);
                }
                for (int k = 0; k < its && rc == SIH_PDHG_OK; ++k) rc = launch_iteration(s);
                if (rc == SIH_PDHG_OK) rc = launch_check(s);
            }
            cudaMemcpyAsync(&h_done[slot], &state_.as<PlainState>()->done, sizeof(int), cudaMemcpyDeviceToHost, s);
            cudaEventRecord(ev[slot], s);
        }
        cudaEventRecord(ev_stop_, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (rc == SIH_PDHG_OK && e != cudaSuccess) rc = cuda_fail(e, "iteration loop", __FILE__, __LINE__);
    }
    for (int w = 0; w < kWindow; ++w)
        if (ev[w]) cudaEventDestroy(ev[w]);
    cudaFreeHost(h_done);
    if (rc != SIH_PDHG_OK) return rc;
    SIHG_CUDA(cudaMemcpy(&host_state_, state_.as<PlainState>(), sizeof(PlainState), cudaMemcpyDeviceToHost));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev_start_, ev_stop_);
    loop_seconds_ = ms * 1e-3;
    return SIH_PDHG_OK;
}

int PlainSolver::fetch(std::vector<float>& best_x, std::vector<float>& y) {
    best_x.resize(hp_->n);
    y.resize(hp_->m);
    SIHG_CUDA(cudaMemcpy(best_x.data(), vec_.best_x, sizeof(float) * hp_->n, cudaMemcpyDeviceToHost));
    SIHG_CUDA(cudaMemcpy(y.data(), vec_.y, sizeof(float) * hp_->m, cudaMemcpyDeviceToHost));
    return SIH_PDHG_OK;
}

PlainSolver::~PlainSolver() {
    if (block_exec_) cudaGraphExecDestroy(block_exec_);
    if (tail_exec_) cudaGraphExecDestroy(tail_exec_);
    if (ev_start_) cudaEventDestroy(ev_start_);
    if (ev_stop_) cudaEventDestroy(ev_stop_);
    if (stream_) cudaStreamDestroy(stream_);
}

}  // namespace sihg
