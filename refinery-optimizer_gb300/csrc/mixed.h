// Mixed-precision restarted adaptive PDHG (scaled, FP32 SpMV, compensated
// reductions with FP64 instance totals)
// for one LP or a batch of LPs; see mixed.cu for the algorithm.
#pragma once

#include <vector>

#include "common.cuh"
#include "host.h"
#include "spmv.cuh"

namespace sihg {

constexpr int kQ = 12;         // reduction slots per task / group
constexpr int kThreads = 256;  // threads per block of every task kernel
constexpr int kStagedThreads = 1024;  // threads per block of the staged step kernels (one block per SM)
constexpr int kGroup = 32;     // tasks per reduction group (one per lane of the reducing warp)
constexpr int kChunk = 2048;   // elements per chunk of the elementwise passes

// Unit of SpMV work of one instance (see warp.cuh): a LIGHT task is the
// contiguous segment range [seg_begin, seg_end) (longer segments skipped); a
// LIST task holds list_idx[seg_begin..seg_end), segments of one length class.
// `flags` bit 0 marks a list task, bits 8..15 hold the lanes per segment.
struct Task {
    int seg_begin;
    int seg_end;
    int inst;
    int flags;
};
constexpr int kTaskList = 1;
__host__ __device__ inline int task_lanes(int flags) { return (flags >> 8) & 0xff; }
constexpr int kTaskSegs = 1024;  // max segments per light task

// Per-instance device state (reduction totals and controller scalars in FP64).
struct Inst {
    // control
    int done;          // 0 running, 1 converged, 2 iteration limit, 3 numerical failure,
                       // 4 converged on the device but above the tolerance in the FP64 check
    int cur;           // buffer holding the current iterate (0 / 1)
    int avg_pending;   // the averages still need the last accepted iterate (weight avg_w)
    int restart_flag;  // set by an evaluation: 0 none, 1 restart at current, 2 restart at average
    int refine;        // compensated (Dot2) evaluation SpMVs
    int out_sel;       // returned point: 0 current, 1 average
    int enable_restart;
    int compensated;   // option: 0 off, 1 near tolerance, 2 always
    long long attempts, steps, rejections, restarts, since_restart, evals, max_attempts;
    // step size and primal weight
    double eta, omega, W, avg_w;
    double kkt_last, kkt_prev;
    // reductions of the current attempt / evaluation
    double dy2;
    double row_eval[8];      // p2[2], pinf[2], dterm[2], dyl2[2]
    double col_eval_dist[2]; // |x_c - x_last|^2
    // last evaluation (index 0 current, 1 average)
    double pobj[2], dobj[2], rel_p[2], rel_d[2], rel_g[2];
    // constants
    double b_inf, c_inf, tol_p, tol_d, tol_g;
    double beta_suff, beta_nec, beta_art, weight_smoothing;
    double kmax, b2, c2;
    double omega_start;  // > 0: initial primal weight of a warm start
    double pow06, pow03; // (attempts + 2)^-0.6 and ^-0.3 of the current attempt
    int verify_rounds;   // times the FP64 check of a converged point sent the instance on
    int pad_;
};

struct Side {
    SegMatrix A;
    const Task* tasks;
    int ntasks;
    const int* list_idx;          // segment ids of the list tasks
    const int* light_max;         // [B] longest segment a light task processes
    const int* task_group;        // [ntasks] reduction group of each task
    const int* group_begin;       // [ngroups + 1] first task of each group
    const int* inst_group_begin;  // [B + 1] first group of each instance
    float2* task_part;            // [ntasks * kQ] task partials (float-float)
    float2* group_part;           // [ngroups * kQ] group partials
    unsigned* group_tickets;      // [ngroups]
    unsigned* tickets;            // [B] completed groups per instance
    unsigned* counters;           // [2] dynamic task counter (zeroed by each compaction), spare
    const int* inst_task_begin;   // [B + 1] first task of each instance
    int* active;                  // [ntasks] tasks of the running instances (rebuilt after evaluations)
    int* nactive;                 // [1] entries of `active`
};

// Chunks of the elementwise passes: {begin, end, instance, is_col}, grouped
// by instance; a chunk never crosses an instance.
struct Chunks {
    const int4* chunks;
    int n;
    const int* inst_begin;  // [B + 1] first chunk of each instance
    int* active;            // [n] chunks of the running instances
    int* nactive;           // [1]
};

// Host-side schedule of one side.
struct SideSchedule {
    std::vector<Task> tasks;
    std::vector<int> list_idx, light_max, task_group, group_begin, inst_group_begin, inst_task_begin;
};

// Host: tasks of every instance of one side (light tasks of at most task_nnz
// light nonzeros, then list tasks per length class) and their reduction groups.
// light_lanes > 0 fixes the lanes per segment of the light tasks (a power of
// two <= 32); 0 picks them from the task's mean segment length.  max_segs caps
// the segments of a light task (at most kTaskSegs).
void make_schedule(const std::vector<int>& ptr, const std::vector<int>& inst_off, int task_nnz, SideSchedule& out,
                   int light_lanes = 0, int max_segs = kTaskSegs);

// Device task layout of a block-diagonal (batched) matrix for the task engine
// (warp.cuh): per side (rows = CSR for A x, columns = CSC for A^T y) the SpMV
// tasks, their reduction groups, partial slots, tickets and active list; the
// element chunks of both sides and their active list (layout.cu).
class TaskLayout {
  public:
    // csr_ptr / csc_ptr: segment pointers of the concatenated matrix (device
    // order); roff / coff: row / column offsets of the instances.  With
    // all_active the active lists hold every task and chunk (no compaction
    // pass needed); otherwise the compaction kernels fill them.
    int build(const std::vector<int>& csr_ptr, const std::vector<int>& csc_ptr, const std::vector<int>& roff,
              const std::vector<int>& coff, const SegMatrix& rows_A, const SegMatrix& cols_A, int task_nnz,
              bool all_active, cudaStream_t s, int row_lanes = 0, int col_lanes = 0, int max_segs = kTaskSegs);

    Side rows{}, cols{};
    Chunks chunks{};
    // 3 x B ints after the three active counts (scratch of the compaction)
    int* compaction_offsets() const { return rows.nactive + 3; }

  private:
    DevMem row_sched_, col_sched_, row_part_, col_part_, tickets_, chunks_, active_;
};

struct Vecs {
    // column side (length N)
    const float *c, *l, *u, *dcol;
    float *x0, *x1, *kty0, *kty1, *x_avg, *x_last, *kty_eval;
    // row side (length M)
    const float *rl, *ru, *drow;
    float *y0, *y1, *kx0, *kx1, *y_avg, *y_last, *kx_eval;
    // step-weighted running averages, accumulated in float-float (hi, lo);
    // x_avg / y_avg above are their FP32 copies, refreshed before every evaluation
    float2 *x_acc, *y_acc;
    // (k^-0.6, k^-0.3) of the step-size schedule for k < pow_n
    const double2* pow_tab;
    int pow_n;
};

class MixedSolver {
  public:
    MixedSolver() = default;
    MixedSolver(const MixedSolver&) = delete;
    MixedSolver& operator=(const MixedSolver&) = delete;
    ~MixedSolver();

    // Concatenates the instances, uploads them, scales them on the device.
    int setup(const std::vector<const HostProblem*>& probs, const sih_pdhg_config& cfg, const sih_pdhg_options& opts);
    // Solves every instance from its initial point until all stop.
    int run();
    // Unscaled primal/dual point returned for instance b (PDHG sign).
    int fetch(int b, std::vector<double>& x, std::vector<double>& y);
    void fill_result(int b, sih_pdhg_result* r) const;

    int instances() const { return B_; }
    double loop_seconds() const { return loop_seconds_; }
    cudaStream_t stream() const { return stream_; }
    const Inst& inst(int b) const { return host_inst_[b]; }
    int launch_step(cudaStream_t s);
    int launch_eval(cudaStream_t s);
    // Times `reps` launches of each step kernel (elementwise, rows, columns).
    int time_kernels(int reps, double* seconds, double* bytes);
    int set_start(int b, const double* x, const double* y, double omega);
    int task_nnz() const { return task_nnz_; }
    bool persistent() const { return persistent_ != 0; }
    // The launch shape in use (autotuner's choice or the rules).
    void launch_shape(sih_pdhg_launch_shape* out) const;
    long long nnz() const { return nnz_; }
    int rows() const { return M_; }
    int cols() const { return N_; }

  private:
    int reset_state();
    int build_schedules(int task_nnz);
    bool latency_bound() const;  // one LP small enough that its steps are latency-bound
    int autotune();
    int launch_compact(cudaStream_t s);
    int record_graph();
    int choose_staging();
    int launch_step_spmvs(cudaStream_t s, int which);
    int launch_persistent(cudaStream_t s, int nsteps);
    int setup_persistent();
    int set_form(int form);
    int setup_packed();
    int apply_shape(const sih_pdhg_launch_shape& sh);
    int time_block(double* seconds);

    std::vector<const HostProblem*> probs_;
    sih_pdhg_config cfg_{};
    sih_pdhg_options opts_{};
    int B_ = 0, M_ = 0, N_ = 0;
    long long nnz_ = 0;
    int sm_count_ = 1;
    int task_nnz_ = 1024;
    int eval_freq_ = 64;
    int grid_ = 1;
    bool timed_out_ = false;
    double loop_seconds_ = 0.0;
    unsigned long long launches_ = 0;  // kernels launched by the last run()
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev_start_ = nullptr, ev_stop_ = nullptr;
    cudaGraphExec_t graphs_[1] = {nullptr};
    std::vector<int> row_off_, col_off_;
    std::vector<int> col_perm_, row_perm_;  // device order -> instance-local original index
    std::vector<int> h_csr_ptr_, h_csc_ptr_;  // segment pointers (device order), for schedule rebuilds
    DevMem csr_ptr_, csc_ptr_, csr_pairs_, csc_pairs_;
    DevMem colvec_, rowvec_, state_, done_count_, accvec_, pow_tab_;
    TaskLayout layout_;
    Side rows_{}, cols_{};
    Chunks chunks_all_{};
    int elem_grid_ = 1;
    // staged gathers (single LP): entries of x (for K x) and of y (for K^T y)
    // copied to shared memory by every block of the step kernels; 0 = off
    int stage_x_ = 0, stage_y_ = 0;
    // persistent step kernel (options.persistent): its grid (every block
    // resident) and the grid barrier's words {arrive, gen, status}
    // (1 = the task-engine form, 2 = the single-LP form with per-block partials)
    int persistent_ = 0, pgrid_ = 0, grid_form1_ = 0, grid_form2_ = 0;
    DevMem bar_, part_, pack_;
    // lanes per segment of the light tasks (0 = length rule), staged prefixes
    // the rule chose (the tuner may switch them off), tuned flag
    int lanes_r_ = 0, lanes_c_ = 0, stage_x_rule_ = 0, stage_y_rule_ = 0, tuned_ = 0;
    int packed_ = 0;  // options.packed: two kernels per step on packed column records
    Vecs V_{};
    std::vector<Inst> host_inst_;
    std::vector<std::vector<float>> start_x_, start_y_;  // warm starts (device order, unscaled)
};

// Runs `rounds` grid barriers of the persistent kernel on a cooperative grid
// of `blocks` blocks that waits for `blocks + missing` arrivals, each wait
// bounded by limit_sec: with missing > 0 every wait runs out.  *timed_out gets
// the barrier's status word, *passed the barriers block 0 passed.
int check_grid_barrier(int blocks, int missing, int rounds, double limit_sec, int* timed_out, int* passed);

int solve_mixed(const HostProblem& hp, const sih_pdhg_config& cfg, const sih_pdhg_options& opts,
                sih_pdhg_result* r);

// H2D bytes of one instance on the mixed path (problem, vectors, renumbering maps).
uint64_t mixed_h2d_bytes(const HostProblem& p);
void pack_solution(const sih_pdhg_problem* p, const sih_pdhg_options& opts, const std::vector<double>& x,
                   const std::vector<double>& y, sih_pdhg_result* r);

}  // namespace sihg
