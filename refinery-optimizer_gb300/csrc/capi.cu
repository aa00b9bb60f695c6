// C-ABI entry points (include/sih_pdhg.h).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>

#include "common.cuh"
#include "host.h"
#include "mixed.h"
#include "plain.h"

namespace sihg {
static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }

bool device_present() {
    int count = 0;
    return cudaGetDeviceCount(&count) == cudaSuccess && count > 0;
}

void clear_result_scalars(sih_pdhg_result* r) {
    r->status = SIH_STATUS_UNKNOWN;
    r->reserved0 = 0;
    r->iterations = 0;
    r->primal_objective = r->dual_bound = 0.0;
    r->rel_primal = r->rel_dual = r->rel_gap = 0.0;
    r->ref_primal = r->ref_dual = 0.0;
    r->time_wall_sec = r->time_solver_sec = 0.0;
    r->restarts = r->step_rejections = 0;
    r->final_step = r->final_primal_weight = 0.0;
    r->h2d_bytes = r->d2h_bytes = 0;
    r->kernel_launches = 0;
}

// Options of an entry point: defaults, or the caller's after a size check.
int resolve_options(const sih_pdhg_options* in, sih_pdhg_options& out) {
    sih_pdhg_options_default(&out);
    if (in) {
        if (in->struct_size != (int32_t)sizeof(sih_pdhg_options))
            return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "options.struct_size does not match this library");
        out = *in;
    }
    if (out.algorithm != SIH_PDHG_ALGO_PLAIN && out.algorithm != SIH_PDHG_ALGO_MIXED)
        return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "unknown algorithm");
    return SIH_PDHG_OK;
}

uint64_t instance_h2d_bytes(const HostProblem& p);

// Fills the vectors and KKT fields of `r` from an FP64 primal/dual pair of
// the internal (minimization) problem; y is in the PDHG sign.
void pack_solution(const sih_pdhg_problem* p, const sih_pdhg_options& opts, const std::vector<double>& x,
                   const std::vector<double>& y, sih_pdhg_result* r) {
    const int64_t m = p->num_rows, n = p->num_cols;
    KktReport k = host_kkt(p, x.data(), y.data(), r->slack, r->reduced_costs);
    // objective and copies: per-thread partials, combined in thread order
    const int T = std::max(1, hardware_threads());
    std::vector<double> part(T, 0.0);
    std::vector<char> fin(2 * (size_t)T, 1);
    parallel_parts(n, T, [&](int64_t b, int64_t e, int t) {
        double o = 0.0;
        bool f = true;
        for (int64_t j = b; j < e; ++j) {
            o += p->c[j] * x[j];
            f = f && std::isfinite(x[j]);
            if (r->x) r->x[j] = x[j];
        }
        part[t] = o;
        fin[t] = f;
    });
    parallel_parts(m, T, [&](int64_t b, int64_t e, int t) {
        bool f = true;
        for (int64_t i = b; i < e; ++i) {
            f = f && std::isfinite(y[i]);
            if (r->row_duals) r->row_duals[i] = opts.dual_sign ? -y[i] * p->sense : y[i];
        }
        fin[T + t] = f;
    });
    double obj = 0.0;
    bool finite = true;
    for (int t = 0; t < T; ++t) obj += part[t];
    for (int t = 0; t < 2 * T; ++t) finite = finite && fin[t];
    r->primal_objective = obj + p->obj_offset;
    r->dual_bound = p->sense * k.dual_obj + p->obj_offset;
    r->rel_primal = k.rel_primal;
    r->rel_dual = k.rel_dual;
    r->rel_gap = k.rel_gap;
    if (!finite) r->status = SIH_STATUS_NUMERICAL_FAILURE;
}

// Packs the result of a plain solver that has iterated.
int solve_plain_packed(PlainSolver& solver, const HostProblem& hp, const sih_pdhg_options& opts, sih_pdhg_result* r) {
    std::vector<float> xf, yf;
    SIHG_TRY(solver.fetch(xf, yf));
    std::vector<double> x(xf.begin(), xf.end()), y(yf.begin(), yf.end());
    r->status = solver.converged() ? SIH_STATUS_OPTIMAL : SIH_STATUS_ITERATION_LIMIT;
    r->iterations = solver.iterations();
    r->ref_primal = solver.last_norm_p();
    r->ref_dual = solver.last_norm_d();
    r->time_solver_sec = solver.loop_seconds();
    r->kernel_launches = solver.launches();
    pack_solution(hp.src, opts, x, y, r);
    r->d2h_bytes = 4ull * (hp.n + hp.m);
    return SIH_PDHG_OK;
}

static int solve_plain(const HostProblem& hp, const sih_pdhg_config& cfg, const sih_pdhg_options& opts,
                       sih_pdhg_result* r) {
    PlainSolver solver;
    SIHG_TRY(solver.setup(hp, cfg, opts));
    SIHG_TRY(solver.iterate());
    SIHG_TRY(solve_plain_packed(solver, hp, opts, r));
    r->h2d_bytes = instance_h2d_bytes(hp);
    return SIH_PDHG_OK;
}

}  // namespace sihg

using namespace sihg;

extern "C" {

int sih_pdhg_abi_version(void) { return SIH_PDHG_ABI_VERSION; }

const char* sih_pdhg_last_error(void) { return g_last_error.c_str(); }

void sih_pdhg_config_default(sih_pdhg_config* c) {
    if (!c) return;
    c->max_iterations = 4000;
    c->tol_primal = 1e-4f;
    c->tol_dual = 1e-4f;
    c->tol_gap = 1e-4f;
    c->check_frequency = 25;
    c->step_tau = 0.0f;
    c->step_sigma = 0.0f;
    c->enable_restart = 1;
    c->enable_hybrid_polish = 1;
}

void sih_pdhg_options_default(sih_pdhg_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->struct_size = (int32_t)sizeof(sih_pdhg_options);
    o->algorithm = SIH_PDHG_ALGO_PLAIN;
    o->ruiz_iterations = 10;
    o->pock_chambolle = 1;
    o->eval_frequency = 64;
    o->compensated = 1;
    o->dual_sign = 0;
    o->use_graph = 1;
    o->reorder = 1;
    o->staged_kib = 0;
    o->autotune = -1;
    o->persistent = -1;
    o->packed = 0;
    o->verbose = 0;
    o->time_limit_sec = 0.0;
    o->restart_sufficient = 0.2;
    o->restart_necessary = 0.8;
    o->restart_artificial = 0.36;
    // PDLP's published 0.5.  Refinery LPs are sensitive to it: FP64 runs of this
    // algorithm on 16 refinery LPs (24 to 168 periods) to 1e-4 took 0.53x the
    // steps in total with 0.8 and 0.50x on the slowest instance, but the FP32
    // engine on the 168-period LP took 15,232 steps with 0.8 against 11,904
    // with 0.5; callers with such LPs can set 0.8 per solve.
    o->primal_weight_smoothing = 0.5;
    o->exact_arithmetic = 0;
    o->lanes_csr = 0;
    o->lanes_csc = 0;
    o->heavy_factor = 16;
}

int sih_pdhg_is_cuda_available(void) { return device_present() ? 1 : 0; }

int sih_pdhg_get_vram_info(uint64_t* total_bytes, uint64_t* free_bytes, uint64_t* used_bytes) {
    if (!device_present()) return fail(SIH_PDHG_ERR_NO_DEVICE, "no CUDA device");
    size_t f = 0, t = 0;
    SIHG_CUDA(cudaMemGetInfo(&f, &t));
    if (total_bytes) *total_bytes = t;
    if (free_bytes) *free_bytes = f;
    if (used_bytes) *used_bytes = t - f;
    return SIH_PDHG_OK;
}

static int solve_ex_impl(const sih_pdhg_problem* problem, const sih_pdhg_config* config, const sih_pdhg_options* opts_in,
                      sih_pdhg_result* result) {
    const auto t0 = std::chrono::steady_clock::now();
    if (!result) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "result is NULL");
    clear_result_scalars(result);
    sih_pdhg_options opts;
    SIHG_TRY(resolve_options(opts_in, opts));
    SIHG_TRY(validate_config(config));
    HostProblem hp;
    SIHG_TRY(build_host_problem(problem, hp));  // validates sizes, pointers and every index
    if (opts.verbose)
        std::fprintf(stderr, "sih_pdhg: host problem %.3f s\n",
                     std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    if (!device_present()) return fail(SIH_PDHG_ERR_NO_DEVICE, "no CUDA device (this engine has no CPU fallback)");
    if (problem->num_rows == 0 || problem->num_cols == 0) {  // gpu_solver.cpp:77-80
        result->status = SIH_STATUS_OPTIMAL;
        for (int64_t j = 0; j < problem->num_cols; ++j)
            if (result->x) result->x[j] = 0.0;
        return SIH_PDHG_OK;
    }
    int rc = opts.algorithm == SIH_PDHG_ALGO_PLAIN ? solve_plain(hp, *config, opts, result)
                                                   : solve_mixed(hp, *config, opts, result);
    result->time_wall_sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int sih_pdhg_solve_ex(const sih_pdhg_problem* problem, const sih_pdhg_config* config, const sih_pdhg_options* opts_in,
                      sih_pdhg_result* result) {
    return guarded([&] { return solve_ex_impl(problem, config, opts_in, result); });
}

int sih_pdhg_solve(const sih_pdhg_problem* problem, const sih_pdhg_config* config, sih_pdhg_result* result) {
    return sih_pdhg_solve_ex(problem, config, nullptr, result);
}

}  // extern "C"
