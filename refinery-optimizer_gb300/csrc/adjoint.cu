// Basis polish and adjoint of the LP solution map, for one LP or a batch.
//
// At a fixed point (x*, y*) of PDHG, the map's Jacobian is fixed by which
// projections are active: a column whose step x - tau (c + A^T y) stays inside
// its bounds moves with the iterate (free), the others sit at a bound; a row
// whose dual prox is clipped is active (its activity equals a bound), the
// others carry no dual.  That pattern is a basis: B = A[active rows, free
// columns], and on it
//     primal   B x_F = b_act - A[act, N] x_N          (x_N at their bounds)
//     dual     B^T lambda = c_F                        (lambda = simplex duals)
//     adjoint  B^T lambda = dL/dx_F:  dL/db_act = lambda,
//              dL/dx_N = g_N - A[act, N]^T lambda (bound of a non-free column),
//              dL/dc = 0 (x* is locally constant in c).
// The pattern is read off a PDHG point: the m variables (columns and row
// slacks) with the largest primal-slack / dual-slack ratio are basic, so B is
// square.  The systems are solved on the GPU by CGLS with the task engine's
// SpMVs on the masked matrix (every instance with its own scalars and stopping
// test; FP32 vectors, compensated reductions, FP64 scalars) inside FP64
// iterative refinement: the residual is recomputed in FP64 on the host and a
// correction solved again, up to four rounds.
//
// The polish (sih_pdhg_polish_batch) returns the basis's vertex and duals:
// from a PDHG point at 1e-6 it recovers the vertex x* whose neighbourhood the
// adjoint differentiates, so a loss evaluated at the polished point has the
// gradient the adjoint returns.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mixed.h"
#include "warp.cuh"

namespace sihg {

struct CgInst {
    int done;    // 0 iterating, 1 converged, 2 iteration limit
    int refine;  // compensated SpMVs (task engine flag; off)
    int init;    // 1 until the first pass has set gamma
    int pad;
    long long iters, max_iters;
    double gamma, alpha, beta, tol2, s0;
};

// CGLS on the masked matrix in one of two orientations.  The UNKNOWN side
// holds z, p, s (mask mu); the RESIDUAL side holds r, q (mask mr).
//   dual (adjoint):  unknown = rows (lambda),  residual = columns
//   primal (polish): unknown = columns (x_F),  residual = rows
struct CgVecs {
    const float *mu, *mr;
    float *z, *p, *s;  // unknown side
    float *r, *q;      // residual side
};

// q = mr .* (K p) over the residual side's segments, |q|^2 -> alpha
struct CgQEpi {
    CgVecs V;
    Acc qq;
    struct Pre {
        float m;
    };
    __device__ Pre pre(int k) const { return Pre{V.mr[k]}; }
    __device__ void begin(const CgInst&) {}
    __device__ const float* gather(int) const { return V.p; }
    __device__ void apply(int k, const SegDot<1>& d, const Pre& pr) {
        const float qv = pr.m * d.f(0);
        V.q[k] = qv;
        qq.add_prod(qv, qv);
    }
    __device__ void values(Acc (&q)[1]) {
        q[0] = qq;
        qq.reset();
    }
    __device__ void finish(CgInst& S, const double* t) { S.alpha = t[0] > 0.0 ? S.gamma / t[0] : 0.0; }
};

// s = mu .* (K^T r) over the unknown side's segments, |s|^2 -> beta, gamma, stop
struct CgSEpi {
    CgVecs V;
    unsigned* done_count;
    double tol;
    Acc ss;
    struct Pre {
        float m;
    };
    __device__ Pre pre(int k) const { return Pre{V.mu[k]}; }
    __device__ void begin(const CgInst&) {}
    __device__ const float* gather(int) const { return V.r; }
    __device__ void apply(int k, const SegDot<1>& d, const Pre& pr) {
        const float sv = pr.m * d.f(0);
        V.s[k] = sv;
        ss.add_prod(sv, sv);
    }
    __device__ void values(Acc (&q)[1]) {
        q[0] = ss;
        ss.reset();
    }
    __device__ void finish(CgInst& S, const double* t) {
        const double v = t[0];
        if (S.init) {
            S.init = 0;
            S.gamma = v;
            S.s0 = v;
            S.beta = 0.0;
            S.tol2 = tol * tol * v;
            if (!(v > 0.0)) {  // right-hand side orthogonal to the basis: zero solution
                S.done = 1;
                atomicAdd(done_count, 1u);
            }
            return;
        }
        S.iters += 1;
        S.beta = S.gamma > 0.0 ? v / S.gamma : 0.0;
        S.gamma = v;
        if (!(v == v)) {
            S.done = 2;
            atomicAdd(done_count, 1u);
        } else if (v <= S.tol2) {
            S.done = 1;
            atomicAdd(done_count, 1u);
        } else if (S.iters >= S.max_iters) {
            S.done = 2;
            atomicAdd(done_count, 1u);
        }
    }
};

__global__ void __launch_bounds__(kThreads) k_cg_q(Side res_side, CgVecs V, CgInst* __restrict__ st) {
    CgQEpi epi{V};
    spmv_engine<1, false, 1>(res_side, st, epi, 0u);
}

__global__ void __launch_bounds__(kThreads) k_cg_s(Side unk_side, CgVecs V, CgInst* __restrict__ st,
                                                   unsigned* done_count, double tol) {
    CgSEpi epi{V, done_count, tol};
    spmv_engine<1, false, 1>(unk_side, st, epi, 0u);
}

// r -= alpha q (residual side), z += alpha p (unknown side)
__global__ void __launch_bounds__(kThreads) k_cg_step(Chunks ch, CgVecs V, CgInst* __restrict__ st, int unk_col) {
    for_each_element(ch, st, [](const CgInst& S) { return (float)S.alpha; }, [&](bool is_col, float a, int k) {
        if (is_col == (unk_col != 0))
            V.z[k] = fmaf(a, V.p[k], V.z[k]);
        else
            V.r[k] = fmaf(-a, V.q[k], V.r[k]);
    });
}

// p = s + beta p (unknown side)
__global__ void __launch_bounds__(kThreads) k_cg_dir(Chunks ch, CgVecs V, CgInst* __restrict__ st, int unk_col) {
    for_each_element(ch, st, [](const CgInst& S) { return (float)S.beta; }, [&](bool is_col, float b, int k) {
        if (is_col == (unk_col != 0)) V.p[k] = fmaf(b, V.p[k], V.s[k]);
    });
}

namespace {

// Basis of one instance from a PDHG point: m basic variables among the n
// columns and m row slacks, by the ratio primal slack / dual slack (in row /
// column norm units).  Equality rows are always active.
struct Basis {
    std::vector<char> free_col, active_row, col_at_lower, row_at_lower;
};

void choose_basis(const sih_pdhg_problem* p, const double* x, const double* y, Basis& B) {
    const int64_t m = p->num_rows, n = p->num_cols;
    std::vector<double> rc(n), ax(m, 0.0), cn(n, 0.0), rn(m, 0.0);
    for (int64_t j = 0; j < n; ++j) {
        double t = 0.0;
        for (int64_t k = p->csc_col_ptr[j]; k < p->csc_col_ptr[j + 1]; ++k) {
            const double a = p->csc_values[k];
            const int64_t i = p->csc_row_ind[k];
            t += a * y[i];
            ax[i] += a * x[j];
            cn[j] += a * a;
            rn[i] += a * a;
        }
        rc[j] = (p->sense == 1 ? p->c[j] : -p->c[j]) + t;  // c + A^T y, PDHG sign
    }
    B.col_at_lower.assign(n, 0);
    B.row_at_lower.assign(m, 0);
    std::vector<std::pair<double, int64_t>> sc((size_t)(n + m));
    auto lg = [](double v) { return std::log(std::max(v, 1e-300)); };
    for (int64_t j = 0; j < n; ++j) {
        const double lo = p->col_lower[j], hi = p->col_upper[j];
        const double dl = bound_is_finite(lo) ? x[j] - lo : INFINITY;
        const double du = bound_is_finite(hi) ? hi - x[j] : INFINITY;
        B.col_at_lower[j] = dl <= du;
        const double ps = std::max(0.0, std::min(dl, du)) * (std::sqrt(cn[j]) + 1e-300);
        sc[j] = {lg(ps) - lg(std::fabs(rc[j])), j};
    }
    for (int64_t i = 0; i < m; ++i) {
        const double lo = p->row_lower[i], hi = p->row_upper[i];
        const double dl = bound_is_finite(lo) ? ax[i] - lo : INFINITY;
        const double du = bound_is_finite(hi) ? hi - ax[i] : INFINITY;
        B.row_at_lower[i] = dl <= du;
        const bool eq = bound_is_finite(lo) && bound_is_finite(hi) && lo == hi;
        const double r = std::sqrt(rn[i]) + 1e-300;
        const double rs = std::max(0.0, std::min(dl, du)) / r;
        sc[n + i] = {eq ? -INFINITY : lg(rs) - lg(std::fabs(y[i]) * r), n + i};
    }
    std::stable_sort(sc.begin(), sc.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    B.free_col.assign(n, 0);
    B.active_row.assign(m, 1);
    for (int64_t k = 0; k < m && k < n + m; ++k) {
        const int64_t id = sc[k].second;
        if (id < n)
            B.free_col[id] = 1;
        else
            B.active_row[id - n] = 0;
    }
}

// Batched masked CGLS on the GPU (both orientations) with FP64 refinement.
class CglsBatch {
  public:
    CglsBatch() = default;
    CglsBatch(const CglsBatch&) = delete;
    CglsBatch& operator=(const CglsBatch&) = delete;
    ~CglsBatch() {
        for (auto& g : graph_)
            if (g) cudaGraphExecDestroy(g);
        if (s_) cudaStreamDestroy(s_);
    }

    int setup(const sih_pdhg_problem* problems, int count, const std::vector<HostProblem>& hps,
              const std::vector<Basis>& basis, const sih_pdhg_adjoint_options& o);
    // Solves (dual) B^T z = rhs [columns, F-masked] or (primal) B z = rhs [rows,
    // R-masked] for every instance; z in FP64 on the unknown side (global
    // order).  iters and status accumulate over calls.
    int solve(bool primal, const std::vector<double>& rhs, std::vector<double>& z);

    std::vector<int> roff, coff;
    std::vector<long long> iters;
    std::vector<double> residual;  // |rhs - B z| / |rhs| (FP64) of the last solve
    std::vector<int> status;       // 0 converged, 1 iteration limit in some round

  private:
    int run_cgls(bool primal, const std::vector<float>& rhs, std::vector<float>& z);
    void product(bool primal, const std::vector<double>& z, std::vector<double>& out) const;

    const sih_pdhg_problem* probs_ = nullptr;
    const std::vector<Basis>* basis_ = nullptr;
    int B_ = 0, M_ = 0, N_ = 0, grid_ = 1, egrid_ = 1;
    long long max_iters_opt_ = 0;
    double tol_ = 1e-6;
    cudaStream_t s_ = nullptr;
    cudaGraphExec_t graph_[2] = {nullptr, nullptr};
    DevMem csr_ptr_, csc_ptr_, csr_, csc_, vec_, state_, done_;
    TaskLayout layout_;
    Side rows_{}, cols_{};
    Chunks ch_{};
    std::vector<float> F_, R_;
    std::vector<int> m_, n_;
};

int CglsBatch::setup(const sih_pdhg_problem* problems, int count, const std::vector<HostProblem>& hps,
                     const std::vector<Basis>& basis, const sih_pdhg_adjoint_options& o) {
    probs_ = problems;
    basis_ = &basis;
    B_ = count;
    tol_ = o.tolerance > 0 ? o.tolerance : 1e-6;
    max_iters_opt_ = o.max_iterations;
    roff.assign(count + 1, 0);
    coff.assign(count + 1, 0);
    m_.resize(count);
    n_.resize(count);
    long long nnz = 0;
    for (int b = 0; b < count; ++b) {
        roff[b + 1] = roff[b] + hps[b].m;
        coff[b + 1] = coff[b] + hps[b].n;
        m_[b] = hps[b].m;
        n_[b] = hps[b].n;
        nnz += hps[b].nnz;
    }
    M_ = roff[count];
    N_ = coff[count];
    if ((long long)M_ >= INT32_MAX - 64 || (long long)N_ >= INT32_MAX - 64 || nnz >= INT32_MAX - 64)
        return fail(SIH_PDHG_ERR_UNSUPPORTED, "batch exceeds the 32-bit index layout");
    std::vector<int> csr_ptr((size_t)M_ + 1), csc_ptr((size_t)N_ + 1);
    PairVec csr((size_t)nnz), csc((size_t)nnz);
    F_.assign(N_, 0.f);
    R_.assign(M_, 0.f);
    std::vector<long long> koff(count + 1, 0);
    for (int b = 0; b < count; ++b) koff[b + 1] = koff[b] + hps[b].nnz;
    parallel_for_min(count, 1, [&](int64_t b0, int64_t b1) {
        for (int64_t b = b0; b < b1; ++b) {
            const HostProblem& hp = hps[b];
            const int ro = roff[b], co = coff[b];
            const long long ko = koff[b];
            for (int i = 0; i < hp.m; ++i) csr_ptr[ro + i] = (int)(hp.csr_ptr[i] + ko);
            for (int j = 0; j < hp.n; ++j) csc_ptr[co + j] = (int)(hp.csc_ptr[j] + ko);
            for (int k = 0; k < hp.nnz; ++k) {
                csr[ko + k] = Pair{hp.csr[k].idx + co, hp.csr[k].val};
                csc[ko + k] = Pair{hp.csc[k].idx + ro, hp.csc[k].val};
            }
            for (int j = 0; j < hp.n; ++j) F_[co + j] = basis[b].free_col[j] ? 1.f : 0.f;
            for (int i = 0; i < hp.m; ++i) R_[ro + i] = basis[b].active_row[i] ? 1.f : 0.f;
        }
    });
    csr_ptr[M_] = (int)nnz;
    csc_ptr[N_] = (int)nnz;

    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count < 1)
        return fail(SIH_PDHG_ERR_NO_DEVICE, "no CUDA device (this engine has no CPU fallback)");
    int dev = 0, sms = 1, occ = 0;
    SIHG_CUDA(cudaGetDevice(&dev));
    SIHG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SIHG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cg_s, kThreads, 0));
    grid_ = sms * std::max(1, occ);
    egrid_ = sms * 4;
    SIHG_CUDA(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
    const int task_nnz =
        (int)std::max(128LL, std::min(2048LL, nnz / std::max(1LL, 3LL * grid_ * (kThreads / 32))));
    auto up = [&](DevMem& d, const void* h, size_t bytes) -> int {
        SIHG_TRY(d.alloc(bytes));
        if (bytes) SIHG_CUDA(cudaMemcpyAsync(d.as<void>(), h, bytes, cudaMemcpyHostToDevice, s_));
        return SIH_PDHG_OK;
    };
    SIHG_TRY(up(csr_ptr_, csr_ptr.data(), sizeof(int) * csr_ptr.size()));
    SIHG_TRY(up(csc_ptr_, csc_ptr.data(), sizeof(int) * csc_ptr.size()));
    SIHG_TRY(up(csr_, csr.data(), sizeof(Pair) * csr.size()));
    SIHG_TRY(up(csc_, csc.data(), sizeof(Pair) * csc.size()));
    // every task and chunk stays listed; a finished instance is skipped by its done flag
    SIHG_TRY(layout_.build(csr_ptr, csc_ptr, roff, coff, SegMatrix{M_, csr_ptr_.as<int>(), csr_.as<int2>()},
                           SegMatrix{N_, csc_ptr_.as<int>(), csc_.as<int2>()}, task_nnz, true, s_));
    rows_ = layout_.rows;
    cols_ = layout_.cols;
    ch_ = layout_.chunks;
    // vectors: F + 3 column vectors, R + 3 row vectors
    SIHG_TRY(vec_.alloc(sizeof(float) * (4 * (size_t)N_ + 4 * (size_t)M_ + 16)));
    float* v = vec_.as<float>();
    SIHG_CUDA(cudaMemcpyAsync(v, F_.data(), sizeof(float) * N_, cudaMemcpyHostToDevice, s_));
    SIHG_CUDA(cudaMemcpyAsync(v + 4 * (size_t)N_, R_.data(), sizeof(float) * M_, cudaMemcpyHostToDevice, s_));
    SIHG_TRY(state_.alloc(sizeof(CgInst) * count));
    SIHG_TRY(done_.alloc(sizeof(unsigned)));
    iters.assign(count, 0);
    residual.assign(count, 0.0);
    status.assign(count, 0);
    return SIH_PDHG_OK;
}

// FP64 product of the masked matrix on the host: primal out[rows] = R .* A (F .* z),
// dual out[cols] = F .* A^T (R .* z).
void CglsBatch::product(bool primal, const std::vector<double>& z, std::vector<double>& out) const {
    out.assign(primal ? M_ : N_, 0.0);
    parallel_for_min(B_, 1, [&](int64_t b0, int64_t b1) {
        for (int64_t b = b0; b < b1; ++b) {
            const sih_pdhg_problem* p = &probs_[b];
            const Basis& bs = (*basis_)[b];
            const int ro = roff[b], co = coff[b];
            for (int64_t j = 0; j < p->num_cols; ++j) {
                if (!bs.free_col[j]) continue;
                if (primal) {
                    const double zj = z[co + j];
                    for (int64_t k = p->csc_col_ptr[j]; k < p->csc_col_ptr[j + 1]; ++k) {
                        const int64_t i = p->csc_row_ind[k];
                        if (bs.active_row[i]) out[ro + i] += p->csc_values[k] * zj;
                    }
                } else {
                    double t = 0.0;
                    for (int64_t k = p->csc_col_ptr[j]; k < p->csc_col_ptr[j + 1]; ++k) {
                        const int64_t i = p->csc_row_ind[k];
                        if (bs.active_row[i]) t += p->csc_values[k] * z[ro + i];
                    }
                    out[co + j] = t;
                }
            }
        }
    });
}

int CglsBatch::run_cgls(bool primal, const std::vector<float>& rhs, std::vector<float>& z) {
    float* v = vec_.as<float>();
    float* c1 = v + N_;                   // three column vectors after F
    float* r1 = v + 4 * (size_t)N_ + M_;  // three row vectors after R
    CgVecs V;
    if (primal)  // unknown = columns, residual = rows
        V = CgVecs{v, v + 4 * (size_t)N_, c1, c1 + N_, c1 + 2 * (size_t)N_, r1, r1 + M_};
    else
        V = CgVecs{v + 4 * (size_t)N_, v, r1, r1 + M_, r1 + 2 * (size_t)M_, c1, c1 + N_};
    const Side& res_side = primal ? rows_ : cols_;
    const Side& unk_side = primal ? cols_ : rows_;
    const int unk_col = primal ? 1 : 0;
    CgInst* st = state_.as<CgInst>();
    unsigned* done = done_.as<unsigned>();
    constexpr int kBlock = 32;
    cudaGraphExec_t& ge = graph_[primal ? 1 : 0];
    if (!ge) {  // CGLS iterations in blocks of 32, one CUDA graph per orientation
        cudaGraph_t g = nullptr;
        SIHG_CUDA(cudaStreamBeginCapture(s_, cudaStreamCaptureModeThreadLocal));
        // the task counters restart with every block (a launch takes a fixed
        // number of counter values, see task_loop)
        cudaError_t e = cudaMemsetAsync(rows_.counters, 0, sizeof(unsigned), s_);
        if (e == cudaSuccess) e = cudaMemsetAsync(cols_.counters, 0, sizeof(unsigned), s_);
        for (int k = 0; k < kBlock && e == cudaSuccess; ++k) {
            k_cg_q<<<grid_, kThreads, 0, s_>>>(res_side, V, st);
            k_cg_step<<<egrid_, kThreads, 0, s_>>>(ch_, V, st, unk_col);
            k_cg_s<<<grid_, kThreads, 0, s_>>>(unk_side, V, st, done, tol_);
            k_cg_dir<<<egrid_, kThreads, 0, s_>>>(ch_, V, st, unk_col);
        }
        const cudaError_t e2 = cudaStreamEndCapture(s_, &g);
        if (e != cudaSuccess) return cuda_fail(e, "graph capture", __FILE__, __LINE__);
        if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture", __FILE__, __LINE__);
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
    }
    const int nres = primal ? M_ : N_, nunk = primal ? N_ : M_;
    SIHG_CUDA(cudaMemcpyAsync(V.r, rhs.data(), sizeof(float) * nres, cudaMemcpyHostToDevice, s_));
    SIHG_CUDA(cudaMemsetAsync(V.q, 0, sizeof(float) * nres, s_));
    SIHG_CUDA(cudaMemsetAsync(V.z, 0, sizeof(float) * 3 * (size_t)nunk, s_));  // z, p, s
    std::vector<CgInst> hst(B_);
    for (int b = 0; b < B_; ++b) {
        std::memset(&hst[b], 0, sizeof(CgInst));
        hst[b].init = 1;
        hst[b].max_iters = max_iters_opt_ > 0 ? max_iters_opt_ : 20LL * (m_[b] + n_[b]) + 1000;
    }
    SIHG_CUDA(cudaMemcpyAsync(st, hst.data(), sizeof(CgInst) * B_, cudaMemcpyHostToDevice, s_));
    SIHG_CUDA(cudaMemsetAsync(done, 0, sizeof(unsigned), s_));
    SIHG_CUDA(cudaMemsetAsync(unk_side.counters, 0, sizeof(unsigned), s_));
    // first pass: s = mu .* K^T r, p = s
    k_cg_s<<<grid_, kThreads, 0, s_>>>(unk_side, V, st, done, tol_);
    k_cg_dir<<<egrid_, kThreads, 0, s_>>>(ch_, V, st, unk_col);
    SIHG_LAUNCH_CHECK();
    long long max_it = 0;
    for (const auto& h : hst) max_it = std::max(max_it, h.max_iters);
    unsigned h_done = 0;
    for (long long it = 0; it < max_it + kBlock; it += kBlock) {
        SIHG_CUDA(cudaMemcpyAsync(&h_done, done, sizeof(unsigned), cudaMemcpyDeviceToHost, s_));
        SIHG_CUDA(cudaStreamSynchronize(s_));
        if ((int)h_done >= B_) break;
        SIHG_CUDA(cudaGraphLaunch(ge, s_));
    }
    z.resize(nunk);
    SIHG_CUDA(cudaMemcpyAsync(z.data(), V.z, sizeof(float) * nunk, cudaMemcpyDeviceToHost, s_));
    SIHG_CUDA(cudaMemcpyAsync(hst.data(), st, sizeof(CgInst) * B_, cudaMemcpyDeviceToHost, s_));
    SIHG_CUDA(cudaStreamSynchronize(s_));
    for (int b = 0; b < B_; ++b) {
        iters[b] += hst[b].iters;
        if (hst[b].done == 2) status[b] = 1;
    }
    return SIH_PDHG_OK;
}

int CglsBatch::solve(bool primal, const std::vector<double>& rhs, std::vector<double>& z) {
    const int nres = primal ? M_ : N_, nunk = primal ? N_ : M_;
    const std::vector<float>& mres = primal ? R_ : F_;
    const std::vector<float>& munk = primal ? F_ : R_;
    const std::vector<int>& ores = primal ? roff : coff;
    z.assign(nunk, 0.0);
    std::vector<double> res(rhs), prod;
    for (int k = 0; k < nres; ++k) res[k] = mres[k] != 0.f ? rhs[k] : 0.0;
    std::vector<double> n0(B_, 0.0), nr(B_, 0.0);
    for (int b = 0; b < B_; ++b)
        for (int k = ores[b]; k < ores[b + 1]; ++k) n0[b] += res[k] * res[k];
    std::vector<float> rf(nres), dz;
    constexpr int kRounds = 4;
    for (int round = 0; round < kRounds; ++round) {
        for (int k = 0; k < nres; ++k) rf[k] = (float)res[k];
        SIHG_TRY(run_cgls(primal, rf, dz));
        for (int k = 0; k < nunk; ++k) z[k] += munk[k] != 0.f ? (double)dz[k] : 0.0;
        product(primal, z, prod);
        bool converged = true;
        for (int b = 0; b < B_; ++b) {
            double s = 0.0;
            for (int k = ores[b]; k < ores[b + 1]; ++k) {
                res[k] = mres[k] != 0.f ? rhs[k] - prod[k] : 0.0;
                s += res[k] * res[k];
            }
            nr[b] = s;
            if (s > 1e-22 * n0[b]) converged = false;
        }
        if (converged) break;
    }
    for (int b = 0; b < B_; ++b) residual[b] = n0[b] > 0.0 ? std::sqrt(nr[b] / n0[b]) : 0.0;
    return SIH_PDHG_OK;
}

int prepare(const sih_pdhg_problem* problems, int count, const double* const* xs, const double* const* ys,
            std::vector<HostProblem>& hps, std::vector<Basis>& basis) {
    hps.resize(count);
    basis.resize(count);
    for (int b = 0; b < count; ++b) {
        SIHG_TRY(build_host_problem(&problems[b], hps[b]));
        if (!xs[b] || !ys[b]) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "NULL x or row_duals");
    }
    parallel_for_min(count, 1, [&](int64_t b0, int64_t b1) {
        for (int64_t b = b0; b < b1; ++b) choose_basis(&problems[b], xs[b], ys[b], basis[b]);
    });
    return SIH_PDHG_OK;
}

double bound_of_row(const sih_pdhg_problem* p, const Basis& bs, int64_t i) {
    const bool eq = p->row_lower[i] == p->row_upper[i];
    return (eq || bs.row_at_lower[i]) ? p->row_lower[i] : p->row_upper[i];
}

}  // namespace
}  // namespace sihg

using namespace sihg;

extern "C" void sih_pdhg_adjoint_options_default(sih_pdhg_adjoint_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->struct_size = (int32_t)sizeof(sih_pdhg_adjoint_options);
    o->tolerance = 1e-6;
    o->max_iterations = 0;
}

static int resolve_adjoint_options(const sih_pdhg_adjoint_options* in, sih_pdhg_adjoint_options& o) {
    sih_pdhg_adjoint_options_default(&o);
    if (in) {
        if (in->struct_size != (int32_t)sizeof(sih_pdhg_adjoint_options))
            return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "adjoint options.struct_size does not match this library");
        o = *in;
    }
    return SIH_PDHG_OK;
}

static int adjoint_batch_impl(const sih_pdhg_problem* problems, int32_t count, const double* const* x,
                                      const double* const* row_duals, const double* const* grad_x,
                                      double* const* grad_c, double* const* grad_row_lower,
                                      double* const* grad_row_upper, double* const* grad_col_lower,
                                      double* const* grad_col_upper, const sih_pdhg_adjoint_options* opts,
                                      sih_pdhg_adjoint_info* info) {
    sih_pdhg_adjoint_options o;
    SIHG_TRY(resolve_adjoint_options(opts, o));
    if (!problems || count < 1 || !x || !row_duals || !grad_x)
        return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "problems, x, row_duals and grad_x are required");
    for (int b = 0; b < count; ++b)
        if (!grad_x[b]) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "NULL grad_x");
    // host part (validation, basis, layout) first, then the device
    std::vector<HostProblem> hps;
    std::vector<Basis> basis;
    SIHG_TRY(prepare(problems, count, x, row_duals, hps, basis));
    CglsBatch cg;
    SIHG_TRY(cg.setup(problems, count, hps, basis, o));
    // B^T lambda = g_F
    std::vector<double> rhs((size_t)cg.coff[count], 0.0), lam;
    for (int b = 0; b < count; ++b)
        for (int64_t j = 0; j < problems[b].num_cols; ++j) rhs[cg.coff[b] + j] = grad_x[b][j];
    SIHG_TRY(cg.solve(false, rhs, lam));
    parallel_for_min(count, 1, [&](int64_t b0, int64_t b1) {
        for (int64_t b = b0; b < b1; ++b) {
            const sih_pdhg_problem* p = &problems[b];
            const Basis& bs = basis[b];
            const int64_t m = p->num_rows, n = p->num_cols;
            const int ro = cg.roff[b];
            for (int64_t i = 0; i < m; ++i) {
                const double li = bs.active_row[i] ? lam[ro + i] : 0.0;
                const bool lo = p->row_lower[i] == p->row_upper[i] || bs.row_at_lower[i];
                if (grad_row_lower && grad_row_lower[b]) grad_row_lower[b][i] = lo ? li : 0.0;
                if (grad_row_upper && grad_row_upper[b]) grad_row_upper[b][i] = lo ? 0.0 : li;
            }
            int64_t nf = 0, na = 0;
            for (int64_t j = 0; j < n; ++j) {
                double t = 0.0;
                for (int64_t k = p->csc_col_ptr[j]; k < p->csc_col_ptr[j + 1]; ++k) {
                    const int64_t i = p->csc_row_ind[k];
                    if (bs.active_row[i]) t += p->csc_values[k] * lam[ro + i];
                }
                const bool fr = bs.free_col[j];
                nf += fr;
                const double gj = fr ? 0.0 : grad_x[b][j] - t;
                if (grad_col_lower && grad_col_lower[b]) grad_col_lower[b][j] = (!fr && bs.col_at_lower[j]) ? gj : 0.0;
                if (grad_col_upper && grad_col_upper[b]) grad_col_upper[b][j] = (!fr && !bs.col_at_lower[j]) ? gj : 0.0;
                if (grad_c && grad_c[b]) grad_c[b][j] = 0.0;
            }
            for (int64_t i = 0; i < m; ++i) na += bs.active_row[i];
            if (info) {
                info[b].status = cg.status[b];
                info[b].reserved = 0;
                info[b].iterations = cg.iters[b];
                info[b].residual = cg.residual[b];
                info[b].free_columns = nf;
                info[b].active_rows = na;
            }
        }
    });
    return SIH_PDHG_OK;
}

extern "C" int sih_pdhg_adjoint_batch(const sih_pdhg_problem* problems, int32_t count, const double* const* x,
                                      const double* const* row_duals, const double* const* grad_x,
                                      double* const* grad_c, double* const* grad_row_lower,
                                      double* const* grad_row_upper, double* const* grad_col_lower,
                                      double* const* grad_col_upper, const sih_pdhg_adjoint_options* opts,
                                      sih_pdhg_adjoint_info* info) {
    return guarded([&] {
        return adjoint_batch_impl(problems, count, x, row_duals, grad_x, grad_c, grad_row_lower, grad_row_upper,
                                  grad_col_lower, grad_col_upper, opts, info);
    });
}

static int polish_batch_impl(const sih_pdhg_problem* problems, int32_t count, const double* const* x,
                                     const double* const* row_duals, double* const* x_out,
                                     double* const* row_duals_out, const sih_pdhg_adjoint_options* opts,
                                     sih_pdhg_polish_info* info) {
    sih_pdhg_adjoint_options o;
    SIHG_TRY(resolve_adjoint_options(opts, o));
    if (!problems || count < 1 || !x || !row_duals || !x_out || !row_duals_out)
        return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "problems, x, row_duals, x_out and row_duals_out are required");
    for (int b = 0; b < count; ++b)
        if (!x_out[b] || !row_duals_out[b]) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "NULL output array");
    std::vector<HostProblem> hps;
    std::vector<Basis> basis;
    SIHG_TRY(prepare(problems, count, x, row_duals, hps, basis));
    CglsBatch cg;
    SIHG_TRY(cg.setup(problems, count, hps, basis, o));
    const int M = cg.roff[count], N = cg.coff[count];
    // primal: B x_F = b_act - A[act, N] x_N, the non-free columns at their bounds
    std::vector<double> xn((size_t)N, 0.0), rhs((size_t)M, 0.0), xf, cf((size_t)N, 0.0), lam;
    parallel_for_min(count, 1, [&](int64_t b0, int64_t b1) {
        for (int64_t b = b0; b < b1; ++b) {
            const sih_pdhg_problem* p = &problems[b];
            const Basis& bs = basis[b];
            const int ro = cg.roff[b], co = cg.coff[b];
            for (int64_t j = 0; j < p->num_cols; ++j) {
                if (bs.free_col[j]) {
                    cf[co + j] = p->sense == 1 ? p->c[j] : -p->c[j];
                    continue;
                }
                const double bound = bs.col_at_lower[j] ? p->col_lower[j] : p->col_upper[j];
                xn[co + j] = bound_is_finite(bound) ? bound : 0.0;
            }
            for (int64_t i = 0; i < p->num_rows; ++i)
                rhs[ro + i] = bs.active_row[i] ? bound_of_row(p, bs, i) : 0.0;
            for (int64_t j = 0; j < p->num_cols; ++j) {
                if (bs.free_col[j] || xn[co + j] == 0.0) continue;
                for (int64_t k = p->csc_col_ptr[j]; k < p->csc_col_ptr[j + 1]; ++k) {
                    const int64_t i = p->csc_row_ind[k];
                    if (bs.active_row[i]) rhs[ro + i] -= p->csc_values[k] * xn[co + j];
                }
            }
        }
    });
    SIHG_TRY(cg.solve(true, rhs, xf));
    const std::vector<double> res_p(cg.residual);
    // dual: B^T lambda = c_F (simplex duals of the internal minimisation)
    SIHG_TRY(cg.solve(false, cf, lam));
    parallel_for_min(count, 1, [&](int64_t b0, int64_t b1) {
        for (int64_t b = b0; b < b1; ++b) {
            const sih_pdhg_problem* p = &problems[b];
            const Basis& bs = basis[b];
            const int64_t m = p->num_rows, n = p->num_cols;
            const int ro = cg.roff[b], co = cg.coff[b];
            double pviol = 0.0, dviol = 0.0, xs = 1.0, cs = 1.0;
            std::vector<double> ax(m, 0.0);
            for (int64_t j = 0; j < n; ++j) {
                const double xj = bs.free_col[j] ? xf[co + j] : xn[co + j];
                x_out[b][j] = xj;
                xs = std::max(xs, std::fabs(xj));
                for (int64_t k = p->csc_col_ptr[j]; k < p->csc_col_ptr[j + 1]; ++k)
                    ax[p->csc_row_ind[k]] += p->csc_values[k] * xj;
                if (bound_is_finite(p->col_lower[j])) pviol = std::max(pviol, p->col_lower[j] - xj);
                if (bound_is_finite(p->col_upper[j])) pviol = std::max(pviol, xj - p->col_upper[j]);
            }
            for (int64_t i = 0; i < m; ++i) {
                if (bound_is_finite(p->row_lower[i])) pviol = std::max(pviol, p->row_lower[i] - ax[i]);
                if (bound_is_finite(p->row_upper[i])) pviol = std::max(pviol, ax[i] - p->row_upper[i]);
                // PDHG sign, as returned with dual_sign 0: y = -lambda
                row_duals_out[b][i] = bs.active_row[i] ? -lam[ro + i] : 0.0;
            }
            // dual feasibility: reduced costs of non-free columns point away
            // from their bounds, row duals have the sign of their active bound
            for (int64_t j = 0; j < n; ++j) {
                const double cj = p->sense == 1 ? p->c[j] : -p->c[j];
                cs = std::max(cs, std::fabs(cj));
                if (bs.free_col[j]) continue;
                double t = 0.0;
                for (int64_t k = p->csc_col_ptr[j]; k < p->csc_col_ptr[j + 1]; ++k) {
                    const int64_t i = p->csc_row_ind[k];
                    if (bs.active_row[i]) t += p->csc_values[k] * lam[ro + i];
                }
                const double rc = cj - t;
                const bool lo_fin = bound_is_finite(p->col_lower[j]), hi_fin = bound_is_finite(p->col_upper[j]);
                if (bs.col_at_lower[j] && lo_fin)
                    dviol = std::max(dviol, -rc);
                else if (!bs.col_at_lower[j] && hi_fin)
                    dviol = std::max(dviol, rc);
                else
                    dviol = std::max(dviol, std::fabs(rc));  // free column held at zero
            }
            for (int64_t i = 0; i < m; ++i) {
                if (!bs.active_row[i] || p->row_lower[i] == p->row_upper[i]) continue;
                const double li = lam[ro + i];
                dviol = std::max(dviol, bs.row_at_lower[i] ? -li : li);
            }
            if (info) {
                info[b].status = cg.status[b];
                info[b].reserved = 0;
                info[b].iterations = cg.iters[b];
                info[b].primal_residual = res_p[b];
                info[b].dual_residual = cg.residual[b];
                info[b].primal_violation = pviol / xs;
                info[b].dual_violation = dviol / cs;
                int64_t nf = 0, na = 0;
                for (int64_t j = 0; j < n; ++j) nf += bs.free_col[j];
                for (int64_t i = 0; i < m; ++i) na += bs.active_row[i];
                info[b].free_columns = nf;
                info[b].active_rows = na;
            }
        }
    });
    return SIH_PDHG_OK;
}

extern "C" int sih_pdhg_polish_batch(const sih_pdhg_problem* problems, int32_t count, const double* const* x,
                                     const double* const* row_duals, double* const* x_out,
                                     double* const* row_duals_out, const sih_pdhg_adjoint_options* opts,
                                     sih_pdhg_polish_info* info) {
    return guarded([&] { return polish_batch_impl(problems, count, x, row_duals, x_out, row_duals_out, opts, info); });
}
