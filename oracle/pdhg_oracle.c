/*
 * CPU oracle for the GPU PDHG path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is a plain-C restatement of the reference's GPU PDHG solve.  It is
 * the reference the CUDA path is compared against (tests, smoke check) and
 * the CPU baseline that the benchmark times beside it.  Nothing in the shipped
 * library links, loads or calls it.
 *
 * What it restates, with citations into the reference project:
 *   - host problem preparation   core/src/gpu/gpu_solver.cpp:82-151
 *       (FP64 -> FP32 casts, CSC -> CSR rebuild in column order, max|c|, max|b|
 *        over finite bounds, diagonal steps 0.95 / max(1, sum |a|))
 *   - initial point              gpu_solver.cpp:192-196, 214-216
 *   - iteration loop             gpu_solver.cpp:227-271
 *   - kernels                    core/src/gpu/cuda_pdhg.cu:14-151
 *       csr_spmv :14-30, csc_spmv :33-49, primal_update :54-77,
 *       dual_update :82-103, restart :106-111, row/col residuals :114-151
 *   - result packing             gpu_solver.cpp:290-304
 * with ONE deliberate difference: the CSC indices are converted to 32-bit
 * integers element by element.  The reference copies its int64 CSC arrays
 * into int32 device buffers byte-for-byte (gpu_solver.cpp:202-203), which
 * corrupts A^T y; the restatement follows the reference's intended math.
 *
 * Floating-point contract: every kernel body is evaluated in float with the
 * same operation order as the reference kernels, and this file is compiled
 * with -ffp-contract=off so that no multiply-add is fused.
 *
 * oracle_kkt() is the FP64 KKT certificate (relative primal residual, dual
 * residual and duality gap as defined in docs/gpu_pdhg.md:51-57, with bound
 * handling of the checker in core/src/checker/checker.cpp:144-235).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Same field order and types as sih::gpu::GpuPdhgConfig (gpu_solver.hpp:12-22). */
typedef struct {
    int32_t max_iterations;
    float tol_primal;
    float tol_dual;
    float tol_gap;
    int32_t check_frequency;
    float step_tau;
    float step_sigma;
    uint8_t enable_restart;
    uint8_t enable_hybrid_polish;
} oracle_config;

typedef struct {
    int32_t status;        /* 0 optimal, 4 iteration limit (SolutionStatus values) */
    int64_t iterations;    /* Solution::simplex_iterations */
    double primal_objective;
    float last_norm_p;     /* reference primal measure at the last check */
    float last_norm_d;     /* reference dual measure at the last check */
    float best_combined;
    int64_t checks;
} oracle_plain_info;

static float maxf_ref(float a, float b) { return (a < b) ? b : a; } /* std::max */
static int finite_bound_d(double v) { return !isinf(v) && fabs(v) < 1e20; } /* is_bounded_*, problem.hpp:29-35 */
static float minf_ref(float a, float b) { return (b < a) ? b : a; } /* std::min */

/* cuda_pdhg.cu:14-30 */
static void csr_spmv(int m, const int* rp, const int* ci, const float* v, const float* x, float* y) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
        float sum = 0.0f;
        for (int k = rp[i]; k < rp[i + 1]; ++k) sum += v[k] * x[ci[k]];
        y[i] = sum;
    }
}

/* cuda_pdhg.cu:33-49 */
static void csc_spmv(int n, const int* cp, const int* ri, const float* v, const float* y, float* z) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j) {
        float sum = 0.0f;
        for (int k = cp[j]; k < cp[j + 1]; ++k) sum += v[k] * y[ri[k]];
        z[j] = sum;
    }
}

/* cuda_pdhg.cu:54-77 */
static void primal_update(int n, const float* tau, const float* c, const float* aty, const float* l,
                          const float* u, float* x, float* xbar) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j) {
        float x_old = x[j];
        float grad = c[j] + aty[j];
        float step = tau[j];
        float x_new = x_old - step * grad;
        float low = l[j], upp = u[j];
        if (x_new < low) x_new = low;
        if (x_new > upp) x_new = upp;
        x[j] = x_new;
        xbar[j] = 2.0f * x_new - x_old;
    }
}

/* cuda_pdhg.cu:82-103 */
static void dual_update(int m, const float* sigma, const float* axbar, const float* rl, const float* ru,
                        float* y) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
        float sig = sigma[i];
        float w = axbar[i] + (y[i] / sig);
        float p = w;
        if (p < rl[i]) p = rl[i];
        if (p > ru[i]) p = ru[i];
        y[i] = sig * (w - p);
    }
}

/* cuda_pdhg.cu:114-129 followed by the host max of gpu_solver.cpp:252-253 */
static float max_row_violation(int m, const float* ax, const float* rl, const float* ru) {
    float best = 0.0f;
#pragma omp parallel
    {
        float local = 0.0f;
#pragma omp for schedule(static)
        for (int i = 0; i < m; ++i) {
            float a = ax[i], viol = 0.0f;
            if (rl[i] > -1e15f && a < rl[i]) viol = fmaxf(viol, rl[i] - a);
            if (ru[i] < 1e15f && a > ru[i]) viol = fmaxf(viol, a - ru[i]);
            local = maxf_ref(local, viol);
        }
#pragma omp critical
        best = maxf_ref(best, local);
    }
    return best;
}

/* cuda_pdhg.cu:131-151 followed by the host max of gpu_solver.cpp:254-255 */
static float max_col_violation(int n, const float* x, const float* c, const float* aty, const float* l,
                               const float* u, const float* tau) {
    float best = 0.0f;
#pragma omp parallel
    {
        float local = 0.0f;
#pragma omp for schedule(static)
        for (int j = 0; j < n; ++j) {
            float xj = x[j];
            float grad = c[j] + aty[j];
            float step = tau[j];
            float proj = xj - step * grad;
            if (proj < l[j]) proj = l[j];
            if (proj > u[j]) proj = u[j];
            local = maxf_ref(local, fabsf(xj - proj) / fmaxf(1e-4f, step));
        }
#pragma omp critical
        best = maxf_ref(best, local);
    }
    return best;
}

/*
 * Reference-semantics plain FP32 PDHG.  Inputs are the reference Problem's
 * int64 CSC arrays and float64 vectors.  Outputs: x_out[n] (best iterate, as
 * double), y_out[m] (last dual, PDHG sign), and *info.  Returns 0, or -1 on an
 * invalid argument.  threads <= 0 keeps the OpenMP default.
 */
int oracle_plain_pdhg(int64_t m64, int64_t n64, const int64_t* cp64, const int64_t* ri64, const double* cv,
                      const double* c64, const double* l64, const double* u64, const double* rl64,
                      const double* ru64, const oracle_config* cfg, double* x_out, double* y_out,
                      oracle_plain_info* info, int threads) {
    if (!cfg || !info || m64 < 0 || n64 < 0 || cfg->check_frequency <= 0) return -1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    memset(info, 0, sizeof(*info));
    const int m = (int)m64, n = (int)n64;
    if (m == 0 || n == 0) { /* gpu_solver.cpp:77-80 */
        info->status = 0;
        return 0;
    }
    const int nnz = (int)cp64[n];

    int* cp = malloc(sizeof(int) * (n + 1));
    int* ri = malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    float* cvf = malloc(sizeof(float) * (nnz > 0 ? nnz : 1));
    for (int j = 0; j <= n; ++j) cp[j] = (int)cp64[j];
    for (int k = 0; k < nnz; ++k) { ri[k] = (int)ri64[k]; cvf[k] = (float)cv[k]; }

    /* CSR rebuild in column order (gpu_solver.cpp:91-109) */
    int* rp = calloc((size_t)m + 1, sizeof(int));
    int* ci = malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    float* rvf = malloc(sizeof(float) * (nnz > 0 ? nnz : 1));
    for (int k = 0; k < nnz; ++k) if (ri[k] < m) rp[ri[k] + 1]++;
    for (int i = 0; i < m; ++i) rp[i + 1] += rp[i];
    int* fill = malloc(sizeof(int) * (m + 1));
    memcpy(fill, rp, sizeof(int) * (m + 1));
    for (int j = 0; j < n; ++j)
        for (int k = cp[j]; k < cp[j + 1]; ++k) {
            int dest = fill[ri[k]]++;
            ci[dest] = j;
            rvf[dest] = cvf[k];
        }
    free(fill);

    float *c = malloc(sizeof(float) * n), *l = malloc(sizeof(float) * n), *u = malloc(sizeof(float) * n);
    float *rl = malloc(sizeof(float) * m), *ru = malloc(sizeof(float) * m);
    float max_abs_c = 1.0f, max_abs_b = 1.0f; /* gpu_solver.cpp:112-126 */
    for (int j = 0; j < n; ++j) {
        c[j] = (float)c64[j];
        l[j] = (float)l64[j];
        u[j] = (float)u64[j];
        max_abs_c = maxf_ref(max_abs_c, fabsf(c[j]));
    }
    for (int i = 0; i < m; ++i) {
        rl[i] = (float)rl64[i];
        ru[i] = (float)ru64[i];
        if (ru[i] < 1e15f) max_abs_b = maxf_ref(max_abs_b, fabsf(ru[i]));
        if (rl[i] > -1e15f) max_abs_b = maxf_ref(max_abs_b, fabsf(rl[i]));
    }

    float *tau = malloc(sizeof(float) * n), *sigma = malloc(sizeof(float) * m); /* :128-151 */
    for (int j = 0; j < n; ++j) {
        float s = 0.0f;
        for (int k = cp[j]; k < cp[j + 1]; ++k) s += fabsf(cvf[k]);
        tau[j] = cfg->step_tau > 0.0f ? cfg->step_tau : 0.95f / maxf_ref(1.0f, s);
    }
    for (int i = 0; i < m; ++i) {
        float s = 0.0f;
        for (int k = rp[i]; k < rp[i + 1]; ++k) s += fabsf(rvf[k]);
        sigma[i] = cfg->step_sigma > 0.0f ? cfg->step_sigma : 0.95f / maxf_ref(1.0f, s);
    }

    float *x = malloc(sizeof(float) * n), *xbar = malloc(sizeof(float) * n), *y = calloc(m, sizeof(float));
    float *aty = malloc(sizeof(float) * n), *axbar = malloc(sizeof(float) * m), *ax = malloc(sizeof(float) * m);
    float* best_x = malloc(sizeof(float) * n);
    for (int j = 0; j < n; ++j) {
        x[j] = maxf_ref(l[j], minf_ref(u[j], 0.0f));
        xbar[j] = x[j];
        best_x[j] = x[j];
    }

    int iter, converged = 0;
    float best_combined = 1e30f;
    for (iter = 1; iter <= cfg->max_iterations; ++iter) {
        csc_spmv(n, cp, ri, cvf, y, aty);
        primal_update(n, tau, c, aty, l, u, x, xbar);
        csr_spmv(m, rp, ci, rvf, xbar, axbar);
        dual_update(m, sigma, axbar, rl, ru, y);
        if (cfg->enable_restart && (iter % 250 == 0)) memcpy(xbar, x, sizeof(float) * n);
        if (iter % cfg->check_frequency == 0 || iter == cfg->max_iterations) {
            csr_spmv(m, rp, ci, rvf, x, ax);
            csc_spmv(n, cp, ri, cvf, y, aty);
            float max_p = max_row_violation(m, ax, rl, ru);
            float max_d = max_col_violation(n, x, c, aty, l, u, tau);
            float norm_p = max_p / max_abs_b, norm_d = max_d / max_abs_c;
            float combined = maxf_ref(norm_p, norm_d);
            info->checks++;
            info->last_norm_p = norm_p;
            info->last_norm_d = norm_d;
            if (combined < best_combined) {
                best_combined = combined;
                memcpy(best_x, x, sizeof(float) * n);
            }
            if (norm_p <= cfg->tol_primal && norm_d <= cfg->tol_dual) {
                converged = 1;
                break;
            }
        }
    }

    info->status = converged ? 0 : 4;
    info->iterations = iter;
    info->best_combined = best_combined;
    double obj = 0.0;
    for (int j = 0; j < n; ++j) {
        if (x_out) x_out[j] = (double)best_x[j];
        obj += c64[j] * (double)best_x[j];
    }
    if (y_out)
        for (int i = 0; i < m; ++i) y_out[i] = (double)y[i];
    info->primal_objective = obj;

    free(cp); free(ri); free(cvf); free(rp); free(ci); free(rvf);
    free(c); free(l); free(u); free(rl); free(ru); free(tau); free(sigma);
    free(x); free(xbar); free(y); free(aty); free(axbar); free(ax); free(best_x);
    return 0;
}

/*
 * Per-iteration timing helper for the CPU baseline: runs exactly `iters`
 * plain PDHG iterations (no checks) on already-converted FP32 data.  Returns
 * 0.  The data layout is the oracle's own (int32 CSR and CSC, float vectors).
 */
int oracle_plain_iterations(int m, int n, const int* cp, const int* ri, const float* cvf, const int* rp,
                            const int* ci, const float* rvf, const float* c, const float* l, const float* u,
                            const float* rl, const float* ru, const float* tau, const float* sigma, float* x,
                            float* xbar, float* y, float* aty, float* axbar, int iters, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    for (int it = 0; it < iters; ++it) {
        csc_spmv(n, cp, ri, cvf, y, aty);
        primal_update(n, tau, c, aty, l, u, x, xbar);
        csr_spmv(m, rp, ci, rvf, xbar, axbar);
        dual_update(m, sigma, axbar, rl, ru, y);
    }
    return 0;
}

/*
 * The reference algorithm solved to a relative-KKT tolerance (the CPU arm of
 * the benchmark).  Each iteration is the four kernels of cuda_pdhg.cu:14-103
 * run as two fused OpenMP passes -- A^T y with the primal update, A x_bar with
 * the dual update -- with the same float operations in the same order as
 * oracle_plain_iterations (so the same iterates).  Initial point and step
 * sizes as oracle_plain_pdhg (gpu_solver.cpp:128-151, entry-order sums).  The
 * reference's own stopping test is off; every `eval_every` iterations the
 * FP64 relative KKT of the current (x, y) is computed (the definitions of
 * oracle_kkt, FP64 matrix values, OpenMP) and the solve stops when all three
 * terms are <= tol, or after max_iters.  out[0..3] = iterations, rel_p, rel_d,
 * rel_gap.  Returns 0, or -1 on an invalid argument.
 */
static void plain_kkt_f64(int m, int n, const int* cp, const int* ri, const double* cv64, const int* rp,
                          const int* ci, const double* rv64, const double* c64, const double* l64, const double* u64,
                          const double* rl64, const double* ru64, double b_inf, double c_inf, const float* x,
                          const float* y, double* rel) {
    double rp_inf = 0.0, rd_inf = 0.0, pobj = 0.0, dobj = 0.0;
#pragma omp parallel for schedule(static) reduction(max : rp_inf, rd_inf) reduction(+ : dobj)
    for (int i = 0; i < m; ++i) {
        double a = 0.0, r = 0.0;
        for (int k = rp[i]; k < rp[i + 1]; ++k) a += rv64[k] * (double)x[ci[k]];
        if (finite_bound_d(rl64[i]) && a < rl64[i]) r = rl64[i] - a;
        if (finite_bound_d(ru64[i]) && a > ru64[i]) r = a - ru64[i];
        rp_inf = fmax(rp_inf, r);
        const double yi = (double)y[i], yn = yi < 0 ? -yi : 0.0, yp = yi > 0 ? yi : 0.0;
        if (finite_bound_d(rl64[i])) dobj += yn * rl64[i]; else rd_inf = fmax(rd_inf, yn);
        if (finite_bound_d(ru64[i])) dobj -= yp * ru64[i]; else rd_inf = fmax(rd_inf, yp);
    }
#pragma omp parallel for schedule(static) reduction(max : rd_inf) reduction(+ : dobj, pobj)
    for (int j = 0; j < n; ++j) {
        double lam = c64[j];
        for (int k = cp[j]; k < cp[j + 1]; ++k) lam += cv64[k] * (double)y[ri[k]];
        pobj += c64[j] * (double)x[j];
        const double pos = lam > 0 ? lam : 0.0, neg = lam < 0 ? -lam : 0.0;
        double rd = 0.0;
        if (finite_bound_d(l64[j])) dobj += pos * l64[j]; else rd = fmax(rd, pos);
        if (finite_bound_d(u64[j])) dobj -= neg * u64[j]; else rd = fmax(rd, neg);
        rd_inf = fmax(rd_inf, rd);
    }
    rel[0] = rp_inf / (1.0 + b_inf);
    rel[1] = rd_inf / (1.0 + c_inf);
    rel[2] = fabs(pobj - dobj) / (1.0 + fabs(pobj) + fabs(dobj));
}

int oracle_plain_solve_kkt(int m, int n, const int* cp, const int* ri, const float* cvf, const double* cv64,
                           const int* rp, const int* ci, const float* rvf, const double* rv64, const double* c64,
                           const double* l64, const double* u64, const double* rl64, const double* ru64, double tol,
                           int eval_every, int max_iters, int threads, double* out) {
    if (m <= 0 || n <= 0 || eval_every <= 0 || max_iters < 0 || !out) return -1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    float *c = malloc(sizeof(float) * n), *l = malloc(sizeof(float) * n), *u = malloc(sizeof(float) * n);
    float *rl = malloc(sizeof(float) * m), *ru = malloc(sizeof(float) * m);
    float *tau = malloc(sizeof(float) * n), *sigma = malloc(sizeof(float) * m);
    float *x = malloc(sizeof(float) * n), *xbar = malloc(sizeof(float) * n), *y = calloc(m, sizeof(float));
    double b_inf = 0.0, c_inf = 0.0;
    for (int j = 0; j < n; ++j) {
        c[j] = (float)c64[j];
        l[j] = (float)l64[j];
        u[j] = (float)u64[j];
        c_inf = fmax(c_inf, fabs(c64[j]));
        float s = 0.0f;
        for (int k = cp[j]; k < cp[j + 1]; ++k) s += fabsf(cvf[k]);
        tau[j] = 0.95f / maxf_ref(1.0f, s);
        x[j] = maxf_ref(l[j], minf_ref(u[j], 0.0f));
        xbar[j] = x[j];
    }
    for (int i = 0; i < m; ++i) {
        rl[i] = (float)rl64[i];
        ru[i] = (float)ru64[i];
        if (finite_bound_d(rl64[i])) b_inf = fmax(b_inf, fabs(rl64[i]));
        if (finite_bound_d(ru64[i])) b_inf = fmax(b_inf, fabs(ru64[i]));
        float s = 0.0f;
        for (int k = rp[i]; k < rp[i + 1]; ++k) s += fabsf(rvf[k]);
        sigma[i] = 0.95f / maxf_ref(1.0f, s);
    }
    double rel[3] = {INFINITY, INFINITY, INFINITY};
    int it = 0;
    while (it < max_iters) {
        const int stop_at = it + eval_every < max_iters ? it + eval_every : max_iters;
        for (; it < stop_at; ++it) {
#pragma omp parallel
            {
#pragma omp for schedule(static)
                for (int j = 0; j < n; ++j) {  /* csc_spmv + primal_update */
                    float sum = 0.0f;
                    for (int k = cp[j]; k < cp[j + 1]; ++k) sum += cvf[k] * y[ri[k]];
                    const float x_old = x[j];
                    float x_new = x_old - tau[j] * (c[j] + sum);
                    if (x_new < l[j]) x_new = l[j];
                    if (x_new > u[j]) x_new = u[j];
                    x[j] = x_new;
                    xbar[j] = 2.0f * x_new - x_old;
                }
#pragma omp for schedule(static)
                for (int i = 0; i < m; ++i) {  /* csr_spmv + dual_update */
                    float sum = 0.0f;
                    for (int k = rp[i]; k < rp[i + 1]; ++k) sum += rvf[k] * xbar[ci[k]];
                    const float sig = sigma[i];
                    const float w = sum + (y[i] / sig);
                    float p = w;
                    if (p < rl[i]) p = rl[i];
                    if (p > ru[i]) p = ru[i];
                    y[i] = sig * (w - p);
                }
            }
        }
        plain_kkt_f64(m, n, cp, ri, cv64, rp, ci, rv64, c64, l64, u64, rl64, ru64, b_inf, c_inf, x, y, rel);
        if (rel[0] <= tol && rel[1] <= tol && rel[2] <= tol) break;
    }
    out[0] = (double)it;
    out[1] = rel[0];
    out[2] = rel[1];
    out[3] = rel[2];
    free(c); free(l); free(u); free(rl); free(ru); free(tau); free(sigma); free(x); free(xbar); free(y);
    return 0;
}

/* Float SpMV exports so tests can compare single kernels. */
void oracle_csr_spmv_f32(int m, const int* rp, const int* ci, const float* v, const float* x, float* y) {
    csr_spmv(m, rp, ci, v, x, y);
}
void oracle_csc_spmv_f32(int n, const int* cp, const int* ri, const float* v, const float* y, float* z) {
    csc_spmv(n, cp, ri, v, y, z);
}
void oracle_primal_update_f32(int n, const float* tau, const float* c, const float* aty, const float* l,
                              const float* u, float* x, float* xbar) {
    primal_update(n, tau, c, aty, l, u, x, xbar);
}
void oracle_dual_update_f32(int m, const float* sigma, const float* axbar, const float* rl, const float* ru,
                            float* y) {
    dual_update(m, sigma, axbar, rl, ru, y);
}

/*
 * FP64 KKT certificate of (x, y) for min c^T x, rl <= A x <= ru, l <= x <= u.
 * y is in the PDHG sign convention of the reference (y_pdhg = -y_simplex,
 * gpu_solver.cpp:297-298), so the reduced cost is lambda = c + A^T y.
 *   primal residual r_p = A x - proj_[rl,ru](A x)           (inf-norm)
 *   dual residual   r_d = part of lambda that no finite bound can carry
 *   dual objective  D   = sum_i [max(-y_i,0) rl_i - max(y_i,0) ru_i]
 *                        + sum_j [max(lambda_j,0) l_j - max(-lambda_j,0) u_j]
 *                        (terms whose bound is infinite are moved to r_d)
 *   rel_p = |r_p|_inf / (1 + |b|_inf), rel_d = |r_d|_inf / (1 + |c|_inf),
 *   rel_gap = |c^T x - D| / (1 + |c^T x| + |D|)              (docs/gpu_pdhg.md:51-57)
 * A bound is finite when |v| < 1e20 (is_bounded_above/below, problem.hpp:29-35).
 * |b|_inf is taken over the finite row bounds.  out[0..5] = rel_p, rel_d,
 * rel_gap, primal objective, dual objective, |r_p|_inf.
 */
static int finite_bound(double v) { return !isinf(v) && fabs(v) < 1e20; }

void oracle_kkt(int64_t m, int64_t n, const int64_t* cp, const int64_t* ri, const double* cv, const double* c,
                const double* l, const double* u, const double* rl, const double* ru, const double* x,
                const double* y, double* out) {
    double* ax = calloc((size_t)(m > 0 ? m : 1), sizeof(double));
    double pobj = 0.0, dobj = 0.0, rp_inf = 0.0, rd_inf = 0.0, b_inf = 0.0, c_inf = 0.0;
    for (int64_t j = 0; j < n; ++j) {
        double lam = c[j];
        for (int64_t k = cp[j]; k < cp[j + 1]; ++k) {
            ax[ri[k]] += cv[k] * x[j];
            lam += cv[k] * y[ri[k]];
        }
        pobj += c[j] * x[j];
        c_inf = fmax(c_inf, fabs(c[j]));
        double pos = lam > 0 ? lam : 0.0, neg = lam < 0 ? -lam : 0.0, rd = 0.0;
        if (finite_bound(l[j])) dobj += pos * l[j]; else rd = fmax(rd, pos);
        if (finite_bound(u[j])) dobj -= neg * u[j]; else rd = fmax(rd, neg);
        rd_inf = fmax(rd_inf, rd);
    }
    for (int64_t i = 0; i < m; ++i) {
        double a = ax[i], r = 0.0;
        if (finite_bound(rl[i])) { b_inf = fmax(b_inf, fabs(rl[i])); if (a < rl[i]) r = rl[i] - a; }
        if (finite_bound(ru[i])) { b_inf = fmax(b_inf, fabs(ru[i])); if (a > ru[i]) r = a - ru[i]; }
        rp_inf = fmax(rp_inf, r);
        double yn = y[i] < 0 ? -y[i] : 0.0, yp = y[i] > 0 ? y[i] : 0.0;
        if (finite_bound(rl[i])) dobj += yn * rl[i]; else rd_inf = fmax(rd_inf, yn);
        if (finite_bound(ru[i])) dobj -= yp * ru[i]; else rd_inf = fmax(rd_inf, yp);
    }
    out[0] = rp_inf / (1.0 + b_inf);
    out[1] = rd_inf / (1.0 + c_inf);
    out[2] = fabs(pobj - dobj) / (1.0 + fabs(pobj) + fabs(dobj));
    out[3] = pobj;
    out[4] = dobj;
    out[5] = rp_inf;
    free(ax);
}
