// Plain FP32 PDHG (the reference's algorithm) on the device.
#pragma once

#include <vector>

#include "common.cuh"
#include "host.h"
#include "mixed.h"
#include "spmv.cuh"

namespace sihg {

// Device-resident loop state of the plain solver (also mirrored on the host).
struct PlainState {
    int done;            // set by the check that meets both tolerances
    int iterations;      // iteration number of that check
    int next_check;      // iteration number of the next check
    int copy_best;       // the last check improved the best combined residual
    unsigned max_p_bits; // running max of row violations (float bits, >= 0)
    unsigned max_d_bits; // running max of column measures (float bits, >= 0)
    float best_combined;
    float last_norm_p;
    float last_norm_d;
    int checks;
    float max_abs_b;
    float max_abs_c;
    float tol_p;
    float tol_d;
    int check_frequency;
    int max_iterations;
    int refine;          // task-engine flag (compensated SpMVs): always 0 here
};

struct PlainVecs {
    const float *c, *l, *u, *tau, *rl, *ru, *sigma;
    float *x, *xbar, *y, *best_x;
};

class PlainSolver {
  public:
    PlainSolver() = default;
    PlainSolver(const PlainSolver&) = delete;
    PlainSolver& operator=(const PlainSolver&) = delete;
    ~PlainSolver();

    // Uploads the problem, computes step sizes, records the CUDA graphs.
    int setup(const HostProblem& hp, const sih_pdhg_config& cfg, const sih_pdhg_options& opts);
    // Runs the iteration loop from the reference's initial point.
    int iterate();
    // Best checked iterate and last dual (FP32, device -> host).
    int fetch(std::vector<float>& best_x, std::vector<float>& y);

    bool converged() const { return host_state_.done != 0; }
    // Reference semantics: the converging check's iteration, else max_iterations + 1.
    int iterations() const { return host_state_.done ? host_state_.iterations : cfg_.max_iterations + 1; }
    float last_norm_p() const { return host_state_.last_norm_p; }
    float last_norm_d() const { return host_state_.last_norm_d; }
    double loop_seconds() const { return loop_seconds_; }
    unsigned long long launches() const { return launches_; }
    cudaStream_t stream() const { return stream_; }
    int launch_iteration(cudaStream_t s);
    int launch_check(cudaStream_t s);
    const SpmvPlan& plan_csr() const { return plan_csr_; }
    const SpmvPlan& plan_csc() const { return plan_csc_; }

  private:
    int record_graphs();
    int record_block(int iters, cudaGraphExec_t* exec);
    int reset_state();

    const HostProblem* hp_ = nullptr;
    sih_pdhg_config cfg_{};
    sih_pdhg_options opts_{};
    bool exact_ = false;
    int sm_count_ = 1;
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev_start_ = nullptr, ev_stop_ = nullptr;
    cudaGraphExec_t block_exec_ = nullptr, tail_exec_ = nullptr;
    DevMem csc_ptr_, csr_ptr_, csc_pairs_, csr_pairs_, colvec_, rowvec_, state_, heavy_;
    TaskLayout layout_;   // task engine of the fast (non-exact) iteration kernels
    int task_grid_ = 1;
    SegMatrix A_{}, At_{};
    SpmvPlan plan_csr_{}, plan_csc_{};
    PlainVecs vec_{};
    std::vector<float> x0_;
    float max_abs_b_ = 1.f, max_abs_c_ = 1.f;
    double loop_seconds_ = 0.0;
    unsigned long long launches_ = 0;  // kernels launched by the last iterate()
    PlainState host_state_{};
};

}  // namespace sihg
