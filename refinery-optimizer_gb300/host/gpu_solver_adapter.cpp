// Drop-in replacement for the reference's core/src/gpu/gpu_solver.cpp.
//
// Compiled inside the reference project (against its headers
// core/include/sih/gpu/gpu_solver.hpp and core/include/sih/model/*.hpp), this
// file implements sih::gpu::GpuSolver on top of the C ABI of
// include/sih_pdhg.h and links against libsih_pdhg.so instead of
// core/src/gpu/cuda_pdhg.cu.  The pybind layer (core/bindings/pybind_module.cpp)
// and the Python wrappers (py/sih_solver/__init__.py) stay unchanged.
//
// Behaviour relative to the reference:
//   * solve_pdhg runs the same algorithm and fills the same Solution fields
//     (status, x = best checked iterate, row_duals = PDHG dual,
//     primal_objective, time_wall_sec, simplex_iterations), plus slack,
//     reduced_costs and dual_bound; sense and obj_offset are honoured;
//   * without a CUDA device it returns status NumericalFailure with the reason
//     in in_solve_log instead of running the CPU simplex (the engine has no CPU
//     fallback);
//   * solve_hybrid keeps the reference's flow: PDHG, then a basis guessed from
//     the PDHG point (scored and selected on the GPU by sih_pdhg_basis_guess),
//     then the FP64 simplex warm start, then a cold FP64 solve if the warm
//     start does not reach optimality.
#include <sih/gpu/gpu_solver.hpp>
#include <sih/simplex/simplex_solver.hpp>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>
#include <vector>

#include "sih_pdhg.h"

namespace sih {
namespace gpu {

namespace {

model::SolutionStatus to_status(int32_t s) { return static_cast<model::SolutionStatus>(s); }

sih_pdhg_config to_c_config(const GpuPdhgConfig& c) {
    sih_pdhg_config out;
    out.max_iterations = c.max_iterations;
    out.tol_primal = c.tol_primal;
    out.tol_dual = c.tol_dual;
    out.tol_gap = c.tol_gap;
    out.check_frequency = c.check_frequency;
    out.step_tau = c.step_tau;
    out.step_sigma = c.step_sigma;
    out.enable_restart = c.enable_restart ? 1 : 0;
    out.enable_hybrid_polish = c.enable_hybrid_polish ? 1 : 0;
    return out;
}

// The reference Problem already holds CSC and CSR (int64 indices, float64
// values); the engine reads them in place.
sih_pdhg_problem to_c_problem(const model::Problem& p) {
    const auto& A = p.A();
    sih_pdhg_problem q;
    q.num_rows = p.num_rows();
    q.num_cols = p.num_cols();
    q.num_nonzeros = p.num_nonzeros();
    q.csc_col_ptr = A.csc_col_ptr().data();
    q.csc_row_ind = A.csc_row_ind().data();
    q.csc_values = A.csc_values().data();
    q.csr_row_ptr = A.csr_row_ptr().data();
    q.csr_col_ind = A.csr_col_ind().data();
    q.csr_values = A.csr_values().data();
    q.c = p.c().data();
    q.col_lower = p.col_lower().data();
    q.col_upper = p.col_upper().data();
    q.row_lower = p.row_lower().data();
    q.row_upper = p.row_upper().data();
    q.sense = static_cast<int32_t>(p.sense());
    q.obj_offset = p.obj_offset();
    return q;
}

}  // namespace

bool GpuSolver::is_cuda_available() noexcept { return sih_pdhg_is_cuda_available() != 0; }

GpuMemoryInfo GpuSolver::get_vram_info() {
    GpuMemoryInfo info;
    uint64_t t = 0, f = 0, u = 0;
    if (sih_pdhg_get_vram_info(&t, &f, &u) == SIH_PDHG_OK) {
        info.total_bytes = t;
        info.free_bytes = f;
        info.used_bytes = u;
    }
    return info;
}

model::Solution GpuSolver::solve_pdhg(const model::Problem& problem, const GpuPdhgConfig& config) {
    model::Solution sol;
    const int64_t m = problem.num_rows(), n = problem.num_cols();
    sol.x.assign(n, 0.0);
    sol.row_duals.assign(m, 0.0);
    sol.slack.assign(m, 0.0);
    sol.reduced_costs.assign(n, 0.0);
    sih_pdhg_problem q = to_c_problem(problem);
    sih_pdhg_config c = to_c_config(config);
    sih_pdhg_result r{};
    r.x = sol.x.data();
    r.row_duals = sol.row_duals.data();
    r.slack = sol.slack.data();
    r.reduced_costs = sol.reduced_costs.data();
    const int rc = sih_pdhg_solve(&q, &c, &r);
    if (rc != SIH_PDHG_OK) {
        sol.status = model::SolutionStatus::NumericalFailure;
        sol.in_solve_log = sih_pdhg_last_error();
        return sol;
    }
    sol.status = to_status(r.status);
    sol.primal_objective = r.primal_objective;
    sol.dual_bound = r.dual_bound;
    sol.simplex_iterations = r.iterations;
    sol.time_wall_sec = r.time_wall_sec;
    sol.time_solver_sec = r.time_solver_sec;
    return sol;
}

model::Solution GpuSolver::solve_hybrid(const model::Problem& problem, const GpuPdhgConfig& config) {
    const auto t0 = std::chrono::steady_clock::now();
    model::Solution pd = solve_pdhg(problem, config);
    const int64_t m = problem.num_rows(), n = problem.num_cols();
    model::Options polish;
    polish.strategy.algorithm = model::AlgorithmChoice::DualSimplex;
    polish.strategy.presolve = model::PresolveMode::Off;
    polish.strategy.enable_scaling = false;
    polish.log_to_console = false;
    if (pd.status == model::SolutionStatus::NumericalFailure) return pd;
    // Basis guess on the GPU (sih_pdhg_basis_guess): columns (value x) and rows
    // (activity A x, the slack the engine returned) ranked by their distance to
    // the nearest finite bound; the m most interior become basic, the rest sit
    // at their nearer bound (the reference's scoring, gpu_solver.cpp:332-395).
    const sih_pdhg_problem q = to_c_problem(problem);
    std::vector<int8_t> cs(n), rs(m);
    if (sih_pdhg_basis_guess(&q, pd.x.data(), pd.slack.data(), cs.data(), rs.data()) != SIH_PDHG_OK) {
        pd.status = model::SolutionStatus::NumericalFailure;
        pd.in_solve_log = sih_pdhg_last_error();
        return pd;
    }
    std::vector<model::BasisStatus> cb(n), rb(m);
    for (int64_t j = 0; j < n; ++j) cb[j] = static_cast<model::BasisStatus>(cs[j]);
    for (int64_t i = 0; i < m; ++i) rb[i] = static_cast<model::BasisStatus>(rs[i]);
    model::Solution sol = simplex::SimplexSolver::solve_from_basis(problem, cb, rb, polish);
    if (!sol.is_optimal()) sol = simplex::SimplexSolver::solve(problem, polish);
    sol.time_wall_sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return sol;
}

}  // namespace gpu
}  // namespace sih
