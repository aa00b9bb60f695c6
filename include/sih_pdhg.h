/*
 * sih_pdhg.h -- C ABI of the GB300 (sm_103a) PDHG LP engine.
 *
 * Drop-in boundary for the reference's GPU PDHG path (kavinR-11/refinery-optimizer):
 * every entry point below names the reference interface it replaces.  The ABI
 * uses plain pointers, sizes and POD structs only; no C++ or framework types
 * cross it, and no entry point throws.  Every function returns an int status
 * (SIH_PDHG_OK or an SIH_PDHG_ERR_* code); sih_pdhg_last_error() gives the
 * message of the calling thread's last failure.
 *
 * Host pointers are used by the sih_pdhg_solve* / handle entry points; the
 * sih_pdhg_launch_* entry points take DEVICE pointers and a cudaStream_t
 * passed as void* (NULL = the legacy default stream), exactly like the
 * reference's launch_* functions they replace.
 */
#ifndef SIH_PDHG_H
#define SIH_PDHG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SIH_PDHG_ABI_VERSION 2

/* ---- status codes of the ABI ------------------------------------------- */
enum {
    SIH_PDHG_OK = 0,
    SIH_PDHG_ERR_INVALID_ARGUMENT = 1, /* bad size, NULL pointer, malformed CSC/CSR, bad config */
    SIH_PDHG_ERR_NO_DEVICE = 2,        /* no CUDA device: the engine has no CPU fallback */
    SIH_PDHG_ERR_CUDA = 3,             /* a CUDA runtime call or kernel launch failed */
    SIH_PDHG_ERR_OUT_OF_MEMORY = 4,    /* device or pinned-host allocation failed */
    SIH_PDHG_ERR_UNSUPPORTED = 5       /* valid request the library cannot serve (e.g. > 2^31-1 nnz) */
};

/* ---- values of sih::model::SolutionStatus (core/include/sih/model/solution.hpp:11-21) */
enum {
    SIH_STATUS_OPTIMAL = 0,
    SIH_STATUS_INFEASIBLE = 1,
    SIH_STATUS_UNBOUNDED = 2,
    SIH_STATUS_TIME_LIMIT = 3,
    SIH_STATUS_ITERATION_LIMIT = 4,
    SIH_STATUS_NODE_LIMIT = 5,
    SIH_STATUS_NUMERICAL_FAILURE = 6,
    SIH_STATUS_INTERRUPTED = 7,
    SIH_STATUS_UNKNOWN = 8
};

/*
 * Same fields, order, types and defaults as sih::gpu::GpuPdhgConfig
 * (core/include/sih/gpu/gpu_solver.hpp:12-22): int, 3 x float, int,
 * 2 x float, 2 x bool (one byte each).  32 bytes on LP64.
 */
typedef struct sih_pdhg_config {
    int32_t max_iterations;      /* 4000 */
    float tol_primal;            /* 1e-4 */
    float tol_dual;              /* 1e-4 */
    float tol_gap;               /* 1e-4 (used by the mixed algorithm; the reference never reads it) */
    int32_t check_frequency;     /* 25, must be > 0 */
    float step_tau;              /* 0 = automatic */
    float step_sigma;            /* 0 = automatic */
    uint8_t enable_restart;      /* 1 */
    uint8_t enable_hybrid_polish; /* 1 (read only by a hybrid caller, not by the PDHG solve) */
} sih_pdhg_config;

/*
 * One LP as the reference's sih::model::Problem holds it
 * (core/include/sih/model/problem.hpp:37-137, sparse_matrix.hpp:20-77):
 *   minimize sense * (c^T x) + obj_offset   (sense 1 = Minimize, -1 = Maximize)
 *   row_lower <= A x <= row_upper,  col_lower <= x <= col_upper
 * A as CSC with int64 indices and float64 values (required) and optionally as
 * CSR (NULL pointers = built here).  When given, the CSR must hold the same
 * entries with columns ascending within each row (the order of
 * SparseMatrix::from_triplets).  Infinite bounds are +-INFINITY or |v| >= 1e20.
 */
typedef struct sih_pdhg_problem {
    int64_t num_rows;
    int64_t num_cols;
    int64_t num_nonzeros;
    const int64_t* csc_col_ptr; /* [num_cols + 1] */
    const int64_t* csc_row_ind; /* [num_nonzeros] */
    const double* csc_values;   /* [num_nonzeros] */
    const int64_t* csr_row_ptr; /* [num_rows + 1] or NULL */
    const int64_t* csr_col_ind; /* [num_nonzeros] or NULL */
    const double* csr_values;   /* [num_nonzeros] or NULL */
    const double* c;            /* [num_cols] */
    const double* col_lower;    /* [num_cols] */
    const double* col_upper;    /* [num_cols] */
    const double* row_lower;    /* [num_rows] */
    const double* row_upper;    /* [num_rows] */
    int32_t sense;
    double obj_offset;
} sih_pdhg_problem;

/* Algorithms served by sih_pdhg_solve_ex. */
enum {
    SIH_PDHG_ALGO_PLAIN = 0, /* the reference's FP32 PDHG: fixed diagonal steps, its termination test */
    SIH_PDHG_ALGO_MIXED = 1  /* restarted adaptive PDHG: Ruiz + Pock-Chambolle scaling, adaptive step,
                                primal weight, KKT restarts; FP32 SpMV/updates, compensated
                                reductions with FP64 totals */
};

/* Settings of the added entry points.  Fill with sih_pdhg_options_default(). */
typedef struct sih_pdhg_options {
    int32_t struct_size;       /* sizeof(sih_pdhg_options) */
    int32_t algorithm;         /* SIH_PDHG_ALGO_* */
    int32_t ruiz_iterations;   /* mixed: Ruiz passes (10) */
    int32_t pock_chambolle;    /* mixed: 1 = apply the alpha=1 Pock-Chambolle pass */
    int32_t eval_frequency;    /* mixed: iterations between restart/termination checks (64) */
    int32_t compensated;       /* mixed: 0 off, 1 on near tolerance (default), 2 always */
    int32_t dual_sign;         /* 0 = PDHG sign of the reference (row_duals = -simplex duals), 1 = simplex sign */
    int32_t use_graph;         /* 1 = replay iteration blocks as CUDA graphs */
    int32_t autotune;          /* mixed: 1 = at creation, time the step kernels' launch shapes (task size, lanes
                                  per segment of each side, staged gathers, and with persistent < 0 the step
                                  form) on this batch and keep the fastest, once per batch shape (instances,
                                  rows, columns, nonzeros; cached per process); 0 = off; -1 = on for batches
                                  of two or more LPs (default) */
    int32_t verbose;           /* 0 */
    double time_limit_sec;     /* <= 0: none */
    double restart_sufficient; /* mixed: 0.2 */
    double restart_necessary;  /* mixed: 0.8 */
    double restart_artificial; /* mixed: 0.36 */
    double primal_weight_smoothing; /* mixed: 0.5 (PDLP); 0.8 adapts faster (refinery LPs) */
    int32_t exact_arithmetic;  /* plain: 1 = the reference kernels' arithmetic (one thread per row/column,
                                  entry-order sums, no fused multiply-add); results then equal the CPU
                                  restatement bit for bit.  0 = warp-cooperative SpMV with FMA (default) */
    int32_t lanes_csr;         /* threads per row of the A x SpMV (mixed: lanes per row of the light tasks, a
                                  power of two <= 32); 0 = automatic (autotuner or heuristic) */
    int32_t lanes_csc;         /* threads per column of the A^T y SpMV (mixed: as lanes_csr); 0 = automatic */
    int32_t heavy_factor;      /* rows/columns longer than heavy_factor * lanes go to whole warps (16) */
    int32_t tile_nnz;          /* mixed: nonzeros per SpMV task (0 = automatic) */
    int32_t reorder;           /* mixed: 1 = renumber columns and rows by descending length inside each
                                  instance so that the vector entries long segments gather share cache
                                  lines (default); 0 = keep the input order */
    int32_t staged_kib;        /* mixed, single LP: shared memory (KiB per block) that holds the first entries of
                                  a gathered vector, so that gathers of the longest segments of the other side
                                  skip L2; the step SpMVs then run one 1024-thread block per SM.  0 = automatic
                                  (on where the staged entries carry a large share of the nonzeros), -1 = off */
    int32_t persistent;        /* mixed: run the steps between two evaluations as ONE persistent cooperative
                                  kernel, phases separated by grid barriers with bounded waits (for LPs whose
                                  steps are latency-bound).  1 = the same tasks and reductions as the
                                  kernel-per-phase path (bit-identical iterates); 2 = for a single LP, static
                                  task shares with per-block partials reduced by every block (no ticket chain;
                                  deterministic, equal to the other forms up to rounding; a batch runs form 1).
                                  0 = one kernel per phase, replayed as CUDA graphs; -1 = automatic (default):
                                  form 2 for one LP whose matrix fits in half of L2, the autotuner's choice
                                  when it runs, else 0. */
    int32_t packed;            /* mixed, kernels per phase: 1 = two kernels per step, the elementwise primal
                                  step folded into the SpMVs (the lanes that gather x' compute it from a packed
                                  16-byte record per column; the column owners store it); same iterates as the
                                  three-kernel step, but slower where measured (the 16-byte gathers cost more
                                  than the elementwise pass: 500k x 1M LP 0.439 -> 0.516 s, 64 refinery
                                  scenarios 47.9 -> 63.8 s).  0 = three kernels (default); staged gathers are
                                  not used with 1.  The single-LP persistent form always works this way. */
    int32_t reserved2;         /* 0 */
} sih_pdhg_options;

/*
 * Result of one solve.  The caller owns the arrays; any may be NULL.
 * Fields mirror what GpuSolver::solve_pdhg writes into sih::model::Solution
 * (core/src/gpu/gpu_solver.cpp:290-304) plus the fields it leaves empty.
 */
typedef struct sih_pdhg_result {
    double* x;             /* [n]  plain: best checked iterate, as the reference; mixed: returned iterate */
    double* row_duals;     /* [m]  sign per options.dual_sign */
    double* slack;         /* [m]  row activity A x */
    double* reduced_costs; /* [n]  c - A^T y_simplex (original space) */
    int32_t status;        /* SIH_STATUS_* */
    int32_t reserved0;
    int64_t iterations;    /* Solution::simplex_iterations semantics (plain: max_iterations + 1 when not converged) */
    double primal_objective;
    double dual_bound;
    double rel_primal;     /* relative KKT of the returned point, FP64 (docs/gpu_pdhg.md:51-57) */
    double rel_dual;
    double rel_gap;
    double ref_primal;     /* the reference's own termination measures at the last check (plain) */
    double ref_dual;
    double time_wall_sec;
    double time_solver_sec; /* device time of the iteration loop */
    int64_t restarts;
    int64_t step_rejections;
    double final_step;
    double final_primal_weight;
    uint64_t h2d_bytes;     /* host -> device bytes this solve moved (problem upload, start point) */
    uint64_t d2h_bytes;     /* device -> host bytes this solve moved (returned point, status) */
    uint64_t kernel_launches; /* kernels this solve launched (graph nodes counted one by one) */
} sih_pdhg_result;

/* Opaque solver handle: one LP or a batch of LPs resident on the device. */
typedef struct sih_pdhg_handle sih_pdhg_handle;

/* ---- metadata ----------------------------------------------------------- */
int sih_pdhg_abi_version(void);
/* Message of the calling thread's last failed call ("" if none). */
const char* sih_pdhg_last_error(void);
void sih_pdhg_config_default(sih_pdhg_config* cfg);
void sih_pdhg_options_default(sih_pdhg_options* opts);

/* Replaces GpuSolver::is_cuda_available (core/src/gpu/gpu_solver.cpp:42-46).
 * Returns 1 when a CUDA device is visible, else 0. */
int sih_pdhg_is_cuda_available(void);

/* Replaces GpuSolver::get_vram_info (core/src/gpu/gpu_solver.cpp:48-58).
 * On the current device.  Errors: SIH_PDHG_ERR_NO_DEVICE. */
int sih_pdhg_get_vram_info(uint64_t* total_bytes, uint64_t* free_bytes, uint64_t* used_bytes);

/*
 * Replaces GpuSolver::solve_pdhg (core/src/gpu/gpu_solver.cpp:60-307).
 * The reference's FP32 PDHG on the current device: same initial point, step
 * sizes, iteration, termination test, best-iterate rule and Solution fields,
 * computed by sm_103a kernels.  Host buffers in, host buffers out.
 * m == 0 or n == 0 returns OK with status Optimal (gpu_solver.cpp:77-80).
 * No device: returns SIH_PDHG_ERR_NO_DEVICE (the reference fell back to CPU
 * simplex, gpu_solver.cpp:66-71; this engine has no CPU fallback).
 */
int sih_pdhg_solve(const sih_pdhg_problem* problem, const sih_pdhg_config* config, sih_pdhg_result* result);

/* sih_pdhg_solve with the added options (algorithm choice etc.).  opts may be NULL (defaults). */
int sih_pdhg_solve_ex(const sih_pdhg_problem* problem, const sih_pdhg_config* config,
                      const sih_pdhg_options* opts, sih_pdhg_result* result);

/* ---- handle API (problems resident on the device between solves) --------
 * Added entry points with no single counterpart in the reference, which
 * re-uploads the problem on every solve_pdhg call (gpu_solver.cpp:153-216). */

/* Uploads `count` LPs (count >= 1) and prepares them for `opts->algorithm`:
 * mixed = one block-diagonal batch solved by one set of kernels with
 * per-instance state; plain = `count` reference-semantics solvers run one
 * after another.  The problem arrays must stay valid until
 * sih_pdhg_destroy (results are checked against them in FP64). */
int sih_pdhg_create(const sih_pdhg_problem* problems, int32_t count, const sih_pdhg_config* config,
                    const sih_pdhg_options* opts, sih_pdhg_handle** out);
/* Solves every instance from its initial point; iterates stay on the device.
 * Returns after all instances stopped.  *device_seconds (may be NULL) gets the
 * device time of the solve (CUDA events on the handle's stream). */
int sih_pdhg_run(sih_pdhg_handle* h, double* device_seconds);
/* Copies instance `index`'s returned point to the host and fills *result
 * (FP64 KKT packing against the problem data given at creation). */
int sih_pdhg_get_result(sih_pdhg_handle* h, int32_t index, sih_pdhg_result* result);
/* Times `reps` back-to-back launches of each SpMV kernel of the mixed solver
 * with CUDA events on the handle's stream: seconds[0] the elementwise primal
 * step, [1] the A x step (rows), [2] the A^T y step (columns); bytes[0..2] get
 * each kernel's algorithmic bytes per launch.  The state is reset by the next run. */
int sih_pdhg_time_kernels(sih_pdhg_handle* h, int32_t reps, double* seconds, double* bytes);
/* Warm start of instance `index` for the following runs (mixed algorithm): x
 * [n] in the original column order and row_duals [m] (may be NULL: zero) in the
 * convention of the returned row_duals (options.dual_sign); primal_weight > 0
 * also replaces the initial primal weight (e.g. the previous result's
 * final_primal_weight).  x == NULL clears the start.  The re-solve caller of
 * the reference (py/refinery/reoptimization.py:81-150) warm-starts its simplex
 * the same way; the reference PDHG has no warm start. */
int sih_pdhg_set_start(sih_pdhg_handle* h, int32_t index, const double* x, const double* row_duals,
                       double primal_weight);
/* Nonzeros per SpMV task in use (mixed algorithm; the autotuner's choice with
 * options.autotune = 1). */
int sih_pdhg_get_task_nnz(const sih_pdhg_handle* h, int32_t* task_nnz);

/* Launch shape of the mixed solver's step kernels: what the autotuner chose
 * (options.autotune) or the rules gave.  No counterpart in the reference, whose
 * kernels launch with fixed 256-thread blocks (cuda_pdhg.cu:155-203). */
typedef struct sih_pdhg_launch_shape {
    int32_t task_nnz;   /* nonzeros per SpMV task */
    int32_t row_lanes;  /* lanes per row of the A x light tasks (0 = the length rule) */
    int32_t col_lanes;  /* lanes per column of the A^T y light tasks (0 = the length rule) */
    int32_t staged_x;   /* entries of x staged in shared memory for A x (0 = off) */
    int32_t staged_y;   /* entries of y staged for A^T y (0 = off) */
    int32_t persistent; /* step form: 0 kernels per phase (graphs), 1 / 2 persistent (options.persistent) */
    int32_t grid;       /* blocks of the step SpMV launches */
    int32_t tuned;      /* 1 when the autotuner chose the shape */
    int32_t packed;     /* 1: two kernels per step (options.packed) */
    int32_t reserved;
} sih_pdhg_launch_shape;
int sih_pdhg_get_launch_shape(const sih_pdhg_handle* h, sih_pdhg_launch_shape* shape);
void sih_pdhg_destroy(sih_pdhg_handle* h);

/* Self-test of the grid barrier of the persistent step kernel
 * (options.persistent; no counterpart in the reference, whose iteration loop
 * has no device-side waits): `rounds` barriers on a cooperative grid of
 * `blocks` blocks that waits for `blocks + missing` arrivals, every wait
 * bounded by limit_sec (at most 10 s).  With missing > 0 no barrier can
 * complete: each block's wait runs out, the kernel returns, *timed_out gets 1
 * and the device stays usable.  *passed gets the barriers completed. */
int sih_pdhg_check_grid_barrier(int32_t blocks, int32_t missing, int32_t rounds, double limit_sec,
                                int32_t* timed_out, int32_t* passed);

/* One-call batch: create + run + result for each instance + destroy.
 * results[count] (arrays inside each may be NULL). */
int sih_pdhg_solve_batch(const sih_pdhg_problem* problems, int32_t count, const sih_pdhg_config* config,
                         const sih_pdhg_options* opts, sih_pdhg_result* results);

/* ---- kernel launchers (device pointers, int32 indices, float values) -----
 * Same arguments and results as the reference's launchers; the reference
 * driver binds them at core/src/gpu/gpu_solver.cpp:18-40. */

/* Replaces launch_csr_spmv (core/src/gpu/cuda_pdhg.cu:155-161): y = A x, A in CSR. */
int sih_pdhg_launch_csr_spmv(int m, const int* d_row_ptr, const int* d_col_ind, const float* d_values,
                             const float* d_x, float* d_y, void* stream);
/* Replaces launch_csc_spmv (cuda_pdhg.cu:163-169): z = A^T y, A in CSC. */
int sih_pdhg_launch_csc_spmv(int n, const int* d_col_ptr, const int* d_row_ind, const float* d_values,
                             const float* d_y, float* d_z, void* stream);
/* Replaces launch_primal_update (cuda_pdhg.cu:171-177):
 * x <- clip(x - tau (c + A^T y), l, u), x_bar <- 2 x_new - x_old. */
int sih_pdhg_launch_primal_update(int n, const float* d_tau, const float* d_c, const float* d_AT_y,
                                  const float* d_l, const float* d_u, float* d_x, float* d_x_bar, void* stream);
/* Replaces launch_dual_update (cuda_pdhg.cu:179-185):
 * w = A x_bar + y / sigma, y <- sigma (w - clip(w, row_l, row_u)). */
int sih_pdhg_launch_dual_update(int m, const float* d_sigma, const float* d_A_xbar, const float* d_row_l,
                                const float* d_row_u, float* d_y, void* stream);
/* Replaces launch_restart (cuda_pdhg.cu:187-191): x_bar <- x. */
int sih_pdhg_launch_restart(int n, const float* d_x, float* d_x_bar, void* stream);
/* Replaces launch_residuals (cuda_pdhg.cu:193-203): per-row bound violation of A x and
 * per-column |x - clip(x - tau (c + A^T y))| / max(1e-4, tau). */
int sih_pdhg_launch_residuals(int m, int n, const float* d_Ax, const float* d_row_l, const float* d_row_u,
                              float* d_row_viols, const float* d_x, const float* d_c, const float* d_AT_y,
                              const float* d_l, const float* d_u, const float* d_tau, float* d_col_viols,
                              void* stream);

/* ---- hybrid polish: basis guess on the device ------------------------------
 * Replaces the host scoring of GpuSolver::solve_hybrid
 * (core/src/gpu/gpu_solver.cpp:332-395) that feeds SimplexSolver::solve_from_basis:
 * every column (value x_j) and row (activity row_activity_i = (A x)_i) gets the
 * distance to its nearer finite bound (bounds beyond +-1e15 count as absent,
 * distance 1e30); the m candidates with the largest distance are Basic (0),
 * the others AtLower (1) or AtUpper (2), the nearer bound (AtLower on a tie).
 * Candidates are columns then rows; equal distances are taken in that order
 * (a stable descending sort, as the reference's std::sort gives for distinct
 * distances).  Scoring and top-m selection (radix select) run on the GPU;
 * host arrays in and out. */
int sih_pdhg_basis_guess(const sih_pdhg_problem* problem, const double* x, const double* row_activity,
                         int8_t* col_status, int8_t* row_status);

/* ---- adjoint (differentiation of the LP solution map) ---------------------
 * No counterpart in the reference (its docs/gpu_pdhg.md plans a differentiable
 * LP layer; the code has none).  Given solved LPs (x, row_duals as returned by
 * this library with options.dual_sign 0) and the gradient of a loss with
 * respect to x, returns the loss gradient with respect to the objective
 * (zero: an LP solution does not move under small cost changes), the row
 * bounds and the column bounds.  The active pattern of the PDHG fixed point
 * is read off (x, y) as a basis (the m variables with the largest
 * primal-slack / dual-slack ratio) and the adjoint system B^T lambda = dL/dx_F
 * of the active rows and free columns is solved on the GPU by CGLS with the
 * engine's SpMV kernels.  An equality row's gradient goes to grad_row_lower.
 * Each pointer array has `count` entries; any output array may be NULL. */
typedef struct sih_pdhg_adjoint_options {
    int32_t struct_size;     /* sizeof(sih_pdhg_adjoint_options) */
    int32_t reserved;
    double tolerance;        /* CGLS stop: normal-equation residual <= tolerance x its initial value (1e-6) */
    int64_t max_iterations;  /* CGLS iterations per instance; 0 = 20 (m + n) + 1000 */
} sih_pdhg_adjoint_options;

typedef struct sih_pdhg_adjoint_info {
    int32_t status;          /* 0 converged, 1 iteration limit */
    int32_t reserved;
    int64_t iterations;      /* CGLS iterations over all refinement rounds */
    double residual;         /* |dL/dx_F - B^T lambda| / |dL/dx_F| in FP64 after the refinement rounds */
    int64_t free_columns;    /* columns of the basis */
    int64_t active_rows;     /* rows whose slack is non-basic (at a bound) */
} sih_pdhg_adjoint_info;

typedef struct sih_pdhg_polish_info {
    int32_t status;            /* 0 both systems converged, 1 an iteration limit was hit */
    int32_t reserved;
    int64_t iterations;        /* CGLS iterations, both systems */
    double primal_residual;    /* |b_act - B x_F| / |b_act| (FP64) */
    double dual_residual;      /* |c_F - B^T lambda| / |c_F| (FP64) */
    double primal_violation;   /* max bound violation of the vertex (rows and columns) / max(1, |x|_inf) */
    double dual_violation;     /* max wrong-sign reduced cost or row dual / max(1, |c|_inf): 0 = optimal basis */
    int64_t free_columns;
    int64_t active_rows;
} sih_pdhg_polish_info;

void sih_pdhg_adjoint_options_default(sih_pdhg_adjoint_options* opts);
/* Basis polish (the GPU half of the reference's hybrid, gpu_solver.cpp:309-420,
 * which ranks variables by distance to their bounds and hands the basis to the
 * FP64 simplex): the basis read off (x, row_duals) as in sih_pdhg_adjoint_batch,
 * then its vertex x_out (B x_F = b_act - A[act, N] x_N) and its duals
 * row_duals_out (B^T lambda = c_F, PDHG sign as returned with dual_sign 0),
 * both by CGLS on the GPU with FP64 refinement.  info reports the residuals
 * and how far the vertex is from primal / dual feasibility (both zero: the
 * basis is optimal and x_out is an exact optimal vertex). */
int sih_pdhg_polish_batch(const sih_pdhg_problem* problems, int32_t count, const double* const* x,
                          const double* const* row_duals, double* const* x_out, double* const* row_duals_out,
                          const sih_pdhg_adjoint_options* opts, sih_pdhg_polish_info* info);
int sih_pdhg_adjoint_batch(const sih_pdhg_problem* problems, int32_t count, const double* const* x,
                           const double* const* row_duals, const double* const* grad_x, double* const* grad_c,
                           double* const* grad_row_lower, double* const* grad_row_upper,
                           double* const* grad_col_lower, double* const* grad_col_upper,
                           const sih_pdhg_adjoint_options* opts, sih_pdhg_adjoint_info* info);

/* ---- problem ingest: MPS files --------------------------------------------
 * Replaces sih::io::read_mps (core/src/io/mps_io.cpp:63-323) on the way into
 * this engine: same records, same problem (row and column bounds, objective,
 * sense, offset, duplicate entries summed and |a| <= 1e-15 dropped as
 * SparseMatrix::from_triplets does, core/src/model/sparse_matrix.cpp:13-88),
 * with CSC and CSR built in one pass instead of a coordinate map.  Integer
 * markers and BV / UI / LI bounds are counted (the PDHG solve takes the LP
 * relaxation, as the reference's does); a QUADOBJ / QMATRIX section returns
 * SIH_PDHG_ERR_UNSUPPORTED.  Parse errors (a token that is not a number,
 * contradictory bounds) return SIH_PDHG_ERR_INVALID_ARGUMENT with the line or
 * the row / column in the message; the reference throws instead.
 * The handle owns every array; sih_pdhg_mps_view points a sih_pdhg_problem
 * (CSC and CSR filled) into them, valid until sih_pdhg_mps_free. */
typedef struct sih_pdhg_mps sih_pdhg_mps;
int sih_pdhg_read_mps(const char* path, sih_pdhg_mps** out);
int sih_pdhg_read_mps_text(const char* text, size_t length, sih_pdhg_mps** out); /* same, from memory */
int sih_pdhg_mps_view(const sih_pdhg_mps* mps, sih_pdhg_problem* problem, const char** name,
                      int64_t* integer_columns); /* name and integer_columns may be NULL */
void sih_pdhg_mps_free(sih_pdhg_mps* mps);

/* ---- convergence check without allocation ---------------------------------
 * No counterpart in the reference.  For callers that must not allocate device
 * memory while they run (a host that hands every library a fixed device pool
 * up front, or a loop in which the synchronising cudaMalloc / cudaFree calls
 * are not allowed): the reference's convergence measures
 * (core/src/gpu/gpu_solver.cpp:242-259) of a point whose data the caller
 * already holds on the device.  Outputs d_out[0] = max row violation of A x /
 * max_abs_b and d_out[1] = max column measure / max_abs_c (the reference's
 * norm_p, norm_d), computed by the kernels of sih_pdhg_launch_csr_spmv,
 * _csc_spmv and _residuals, with the working arrays in a file-scope device
 * array of the library instead of cudaMalloc: the library calls no
 * cudaMalloc, cudaFree or allocating routine.  `nnz` picks the lane groups as
 * the launchers do.  A NaN measure is skipped, as the reference's host loop
 * skips it.
 * Limit: m + n <= 524,288; larger sizes return SIH_PDHG_ERR_INVALID_ARGUMENT.
 * The array (4 MiB) stays on every GPU that loaded the library until exit.
 * The first call on a device does the set-up: it looks the array's address up
 * with that device current, and CUDA may load the library's device code then
 * (which is when the array itself is placed); make that first call before any
 * stream capture.  Later calls allocate nothing.  After cudaDeviceReset the
 * next call does the set-up again (the context id changed).
 * All calls share the array: calls that overlap on the GPU (other streams,
 * other threads) race and must be serialised by the caller. */
int sih_pdhg_check_norms_noalloc(int m, int n, int nnz, const int* d_row_ptr, const int* d_col_ind,
                                 const float* d_csr_values, const int* d_col_ptr, const int* d_row_ind,
                                 const float* d_csc_values, const float* d_x, const float* d_y, const float* d_c,
                                 const float* d_l, const float* d_u, const float* d_tau, const float* d_row_l,
                                 const float* d_row_u, float max_abs_b, float max_abs_c, float* d_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SIH_PDHG_H */
