/*
 * FP64 CPU oracle of the mixed-precision restarted adaptive PDHG -- TEST
 * INFRASTRUCTURE ONLY (what the CUDA path is compared against; nothing ships it).
 *
 * The reference's GPU path does not implement the adaptive pieces that its
 * own design document asks for (docs/gpu_pdhg.md:42-57: equilibration,
 * normalized termination residuals); this file restates, in double precision
 * and in the same order of operations as the CUDA path, the published method:
 *   - Ruiz equilibration (inf-norm) and one Pock-Chambolle pass (alpha = 1),
 *   - PDLP adaptive step size and primal weight (Applegate et al., NeurIPS
 *     2021, "Practical large-scale linear programming using primal-dual hybrid
 *     gradient", Algorithm 3 and Section 3.3),
 *   - KKT-based adaptive restarts to the current or step-weighted average
 *     iterate (the restart rule of cuPDLP, Lu & Yang 2023, with the PDLP
 *     constants 0.2 / 0.8 / 0.36),
 *   - termination on the relative KKT error of docs/gpu_pdhg.md:51-57.
 * The PDHG sign convention is the reference's (y_pdhg = -simplex dual, dual
 * step y <- sigma (w - clip(w, rl, ru)) as in core/src/gpu/cuda_pdhg.cu:82-103).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int32_t ruiz_iterations, pock_chambolle, eval_frequency, enable_restart;
    int64_t max_attempts;
    double tol_p, tol_d, tol_g;
    double beta_suff, beta_nec, beta_art, weight_smoothing;
    /* FP32 emulation bits: 1 iterates x, y; 2 products K x, K^T y; 4 averages;
       8 scaled data (matrix, c, bounds); 16 average candidates rounded to FP32
       at each evaluation (the averages themselves stay in double).
       0 = everything in double. */
    int32_t fp32_bits;
} pdlp_oracle_opts;

static void round_f(double* v, int n, int on) {
    if (!on) return;
    for (int i = 0; i < n; ++i) v[i] = (double)(float)v[i];
}

typedef struct {
    int32_t status; /* 0 optimal, 4 iteration limit, 6 numerical failure */
    int32_t out_sel;
    int64_t attempts, steps, rejections, restarts, evals;
    double eta, omega, rel_p, rel_d, rel_g, pobj, dobj;
} pdlp_oracle_info;

typedef struct {
    int m, n, nnz;
    int *cp, *ri, *rp, *ci;
    double *cv, *rv; /* scaled values, CSC and CSR */
} mat_t;

static int fin(double v) { return !isinf(v); }
static double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* OpenMP only on loops whose iterations are independent (SpMV rows / columns,
 * elementwise updates): the results equal the one-thread run bit for bit; the
 * reductions stay sequential.  Small LPs run on one thread. */
#define PAR_MIN 50000

static void mat_x(const mat_t* A, const double* x, double* out) {
#pragma omp parallel for schedule(static) if (A->m > PAR_MIN)
    for (int i = 0; i < A->m; ++i) {
        double s = 0.0;
        for (int k = A->rp[i]; k < A->rp[i + 1]; ++k) s += A->rv[k] * x[A->ci[k]];
        out[i] = s;
    }
}
static void mat_ty(const mat_t* A, const double* y, double* out) {
#pragma omp parallel for schedule(static) if (A->n > PAR_MIN)
    for (int j = 0; j < A->n; ++j) {
        double s = 0.0;
        for (int k = A->cp[j]; k < A->cp[j + 1]; ++k) s += A->cv[k] * y[A->ri[k]];
        out[j] = s;
    }
}

/* one scaling pass: mode 0 inf-norm (Ruiz), 1 one-norm (Pock-Chambolle) */
static void scale_pass(mat_t* A, int mode, double* dcol, double* drow, double* fc, double* fr) {
    for (int j = 0; j < A->n; ++j) {
        double acc = 0.0;
        for (int k = A->cp[j]; k < A->cp[j + 1]; ++k) acc = mode == 0 ? fmax(acc, fabs(A->cv[k])) : acc + fabs(A->cv[k]);
        fc[j] = acc > 0.0 ? 1.0 / sqrt(acc) : 1.0;
    }
    for (int i = 0; i < A->m; ++i) {
        double acc = 0.0;
        for (int k = A->rp[i]; k < A->rp[i + 1]; ++k) acc = mode == 0 ? fmax(acc, fabs(A->rv[k])) : acc + fabs(A->rv[k]);
        fr[i] = acc > 0.0 ? 1.0 / sqrt(acc) : 1.0;
    }
    for (int i = 0; i < A->m; ++i)
        for (int k = A->rp[i]; k < A->rp[i + 1]; ++k) A->rv[k] *= fr[i] * fc[A->ci[k]];
    for (int j = 0; j < A->n; ++j)
        for (int k = A->cp[j]; k < A->cp[j + 1]; ++k) A->cv[k] *= fc[j] * fr[A->ri[k]];
    for (int j = 0; j < A->n; ++j) dcol[j] *= fc[j];
    for (int i = 0; i < A->m; ++i) drow[i] *= fr[i];
}

typedef struct {
    double kkt, rel_p, rel_d, rel_g, pobj, dobj, dist_x2, dist_y2;
} cand_eval;

/* KKT of candidate (x, y) with products kx = K x, kty = K^T y (scaled space). */
static cand_eval eval_candidate(const mat_t* A, const double* c, const double* l, const double* u, const double* rl,
                                const double* ru, const double* dcol, const double* drow, const double* x,
                                const double* y, const double* kx, const double* kty, const double* x_last,
                                const double* y_last, double omega, double b_inf, double c_inf) {
    cand_eval e;
    double p2 = 0, pinf = 0, d2 = 0, dinf = 0, pobj = 0, dobj = 0, dx2 = 0, dy2 = 0;
    for (int i = 0; i < A->m; ++i) {
        double res = 0.0;
        if (kx[i] < rl[i]) res = rl[i] - kx[i];
        if (kx[i] > ru[i]) res = kx[i] - ru[i];
        p2 += res * res;
        pinf = fmax(pinf, res / drow[i]);
        if (y[i] < 0 && fin(rl[i])) dobj += -y[i] * rl[i];
        if (y[i] > 0 && fin(ru[i])) dobj -= y[i] * ru[i];
        dy2 += (y[i] - y_last[i]) * (y[i] - y_last[i]);
    }
    for (int j = 0; j < A->n; ++j) {
        const double lam = c[j] + kty[j];
        double rd = 0.0;
        if (lam > 0) {
            if (fin(l[j])) dobj += lam * l[j]; else rd = lam;
        } else if (lam < 0) {
            if (fin(u[j])) dobj += lam * u[j]; else rd = -lam;
        }
        d2 += rd * rd;
        dinf = fmax(dinf, rd / dcol[j]);
        pobj += c[j] * x[j];
        dx2 += (x[j] - x_last[j]) * (x[j] - x_last[j]);
    }
    const double gap = fabs(pobj - dobj);
    e.rel_p = pinf / (1.0 + b_inf);
    e.rel_d = dinf / (1.0 + c_inf);
    e.rel_g = gap / (1.0 + fabs(pobj) + fabs(dobj));
    e.kkt = sqrt(omega * p2 + d2 / omega + gap * gap);
    e.pobj = pobj;
    e.dobj = dobj;
    e.dist_x2 = dx2;
    e.dist_y2 = dy2;
    return e;
}

static int is_inf_bound(double v) { return isinf(v) || fabs(v) >= 1e20; }

/*
 * Solves one LP.  Inputs: int64 CSC + float64 data of the original problem
 * (minimization; a maximization caller negates c).  Outputs: unscaled x[n]
 * and y[m] (PDHG sign) of the returned point, and *info.
 */
int pdlp_oracle_solve(int64_t m64, int64_t n64, const int64_t* cp64, const int64_t* ri64, const double* cv64,
                      const double* c0, const double* l0, const double* u0, const double* rl0, const double* ru0,
                      const pdlp_oracle_opts* o, double* x_out, double* y_out, pdlp_oracle_info* info) {
    const int m = (int)m64, n = (int)n64, nnz = (int)cp64[n];
    memset(info, 0, sizeof(*info));
    mat_t A = {m, n, nnz, malloc(sizeof(int) * (n + 1)), malloc(sizeof(int) * (nnz + 1)),
               calloc(m + 1, sizeof(int)), malloc(sizeof(int) * (nnz + 1)), malloc(sizeof(double) * (nnz + 1)),
               malloc(sizeof(double) * (nnz + 1))};
    for (int j = 0; j <= n; ++j) A.cp[j] = (int)cp64[j];
    for (int k = 0; k < nnz; ++k) { A.ri[k] = (int)ri64[k]; A.cv[k] = cv64[k]; }
    for (int k = 0; k < nnz; ++k) A.rp[A.ri[k] + 1]++;
    for (int i = 0; i < m; ++i) A.rp[i + 1] += A.rp[i];
    int* fill = malloc(sizeof(int) * (m + 1));
    memcpy(fill, A.rp, sizeof(int) * (m + 1));
    for (int j = 0; j < n; ++j)
        for (int k = A.cp[j]; k < A.cp[j + 1]; ++k) {
            const int d = fill[A.ri[k]]++;
            A.ci[d] = j;
            A.rv[d] = A.cv[k];
        }
    free(fill);
    double *c = malloc(8 * n), *l = malloc(8 * n), *u = malloc(8 * n), *dcol = malloc(8 * n), *fc = malloc(8 * n);
    double *rl = malloc(8 * m), *ru = malloc(8 * m), *drow = malloc(8 * m), *fr = malloc(8 * m);
    double b_inf = 0, c_inf = 0;
    for (int j = 0; j < n; ++j) {
        c[j] = c0[j];
        l[j] = is_inf_bound(l0[j]) ? -INFINITY : l0[j];
        u[j] = is_inf_bound(u0[j]) ? INFINITY : u0[j];
        dcol[j] = 1.0;
        c_inf = fmax(c_inf, fabs(c0[j]));
    }
    for (int i = 0; i < m; ++i) {
        rl[i] = is_inf_bound(rl0[i]) ? -INFINITY : rl0[i];
        ru[i] = is_inf_bound(ru0[i]) ? INFINITY : ru0[i];
        drow[i] = 1.0;
        if (fin(rl[i])) b_inf = fmax(b_inf, fabs(rl[i]));
        if (fin(ru[i])) b_inf = fmax(b_inf, fabs(ru[i]));
    }
    for (int k = 0; k < o->ruiz_iterations; ++k) scale_pass(&A, 0, dcol, drow, fc, fr);
    if (o->pock_chambolle) scale_pass(&A, 1, dcol, drow, fc, fr);
    double kmax = 0, b2 = 0, c2 = 0;
    for (int j = 0; j < n; ++j) {
        c[j] *= dcol[j];
        l[j] /= dcol[j];
        u[j] /= dcol[j];
        c2 += c[j] * c[j];
    }
    for (int i = 0; i < m; ++i) {
        rl[i] *= drow[i];
        ru[i] *= drow[i];
        const double b = fin(rl[i]) ? rl[i] : (fin(ru[i]) ? ru[i] : 0.0);
        b2 += b * b;
    }
    if (o->fp32_bits & 8) {
        round_f(A.rv, nnz, 1);
        round_f(A.cv, nnz, 1);
        round_f(c, n, 1);
        round_f(l, n, 1);
        round_f(u, n, 1);
        round_f(rl, m, 1);
        round_f(ru, m, 1);
    }
    for (int k = 0; k < nnz; ++k) kmax = fmax(kmax, fabs(A.rv[k]));
    double eta = kmax > 0 ? 1.0 / kmax : 1.0;
    double omega = (sqrt(c2) > 1e-10 && sqrt(b2) > 1e-10) ? sqrt(c2) / sqrt(b2) : 1.0;

    double *x = malloc(8 * n), *xn = malloc(8 * n), *kty = calloc(n, 8), *ktyn = malloc(8 * n);
    double *x_avg = malloc(8 * n), *x_last = malloc(8 * n), *kty_avg = malloc(8 * n);
    double *y = calloc(m, 8), *yn = malloc(8 * m), *kx = malloc(8 * m), *kxn = malloc(8 * m);
    double *y_avg = calloc(m, 8), *y_last = calloc(m, 8), *kx_avg = malloc(8 * m);
    for (int j = 0; j < n; ++j) x[j] = x_avg[j] = x_last[j] = clampd(0.0, l[j], u[j]);
    mat_x(&A, x, kx);

    double W = 0, kkt_last = 0, kkt_prev = 0;
    int64_t attempts = 0, steps = 0, rejections = 0, restarts = 0, since = 0, evals = 0;
    int status = -1, out_sel = 0;
    const int E = o->eval_frequency > 0 ? o->eval_frequency : 64;
    cand_eval ev[2];
    double* xa_acc = (o->fp32_bits & 16) ? malloc(8 * (n > 0 ? n : 1)) : NULL;
    double* ya_acc = (o->fp32_bits & 16) ? malloc(8 * (m > 0 ? m : 1)) : NULL;
    for (;;) {
        /* ---- evaluation (also at attempt 0) */
        if (xa_acc) { /* candidate = FP32 copy of the FP64 average */
            memcpy(xa_acc, x_avg, 8 * n);
            memcpy(ya_acc, y_avg, 8 * m);
            round_f(x_avg, n, 1);
            round_f(y_avg, m, 1);
        }
        mat_x(&A, x_avg, kx_avg);
        mat_ty(&A, y_avg, kty_avg);
        round_f(kx_avg, m, o->fp32_bits & 2);
        round_f(kty_avg, n, o->fp32_bits & 2);
        {
            /* current candidate: fresh products (the CUDA path recomputes them too) */
            double* kx2 = malloc(8 * (m > 0 ? m : 1));
            double* kty2 = malloc(8 * (n > 0 ? n : 1));
            mat_x(&A, x, kx2);
            mat_ty(&A, y, kty2);
            ev[0] = eval_candidate(&A, c, l, u, rl, ru, dcol, drow, x, y, kx2, kty2, x_last, y_last, omega, b_inf,
                                   c_inf);
            free(kx2);
            free(kty2);
        }
        ev[1] = eval_candidate(&A, c, l, u, rl, ru, dcol, drow, x_avg, y_avg, kx_avg, kty_avg, x_last, y_last, omega,
                               b_inf, c_inf);
        const int have_avg = W > 0.0;
        if (!have_avg) ev[1].kkt = INFINITY;
        evals++;
        if (!(ev[0].kkt == ev[0].kkt)) { status = 6; out_sel = 0; break; }
        int stop = 0;
        for (int cc = 0; cc < 2 && !stop; ++cc) {
            if (cc == 1 && !have_avg) break;
            if (ev[cc].rel_p <= o->tol_p && ev[cc].rel_d <= o->tol_d && ev[cc].rel_g <= o->tol_g) {
                status = 0;
                out_sel = cc;
                stop = 1;
            }
        }
        if (stop) break;
        const int cand = ev[1].kkt < ev[0].kkt ? 1 : 0;
        if (attempts >= o->max_attempts) { status = 4; out_sel = cand; break; }
        const double kc = ev[cand].kkt;
        int restart_flag = 0;
        if (evals == 1) {
            kkt_last = kkt_prev = kc;
            restart_flag = 1;
        } else if (o->enable_restart) {
            const int restart = kc <= o->beta_suff * kkt_last || (kc <= o->beta_nec * kkt_last && kc > kkt_prev) ||
                                (double)since >= o->beta_art * (double)steps;
            kkt_prev = kc;
            if (restart) {
                const double dxn = sqrt(ev[cand].dist_x2), dyn = sqrt(ev[cand].dist_y2);
                if (dxn > 1e-10 && dyn > 1e-10)
                    omega = exp(o->weight_smoothing * log(dyn / dxn) + (1.0 - o->weight_smoothing) * log(omega));
                kkt_last = kc;
                restart_flag = cand == 1 ? 2 : 1;
                restarts++;
                since = 0;
                W = 0.0;
            }
        }
        if (xa_acc && restart_flag == 0) { /* keep accumulating in double unless a restart replaced it */
            memcpy(x_avg, xa_acc, 8 * n);
            memcpy(y_avg, ya_acc, 8 * m);
        }
        if (restart_flag == 2) {
            memcpy(x, x_avg, 8 * n);
            memcpy(kty, kty_avg, 8 * n);
            memcpy(y, y_avg, 8 * m);
            memcpy(kx, kx_avg, 8 * m);
        }
        if (restart_flag) {
            memcpy(x_last, x, 8 * n);
            memcpy(y_last, y, 8 * m);
        }
        /* ---- E attempts */
        for (int a = 0; a < E; ++a) {
            const double tau = eta / omega, sigma = eta * omega;
            double dx2 = 0, dy2 = 0, inter = 0;
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
            for (int j = 0; j < n; ++j) xn[j] = clampd(x[j] - tau * (c[j] + kty[j]), l[j], u[j]);
            round_f(xn, n, o->fp32_bits & 1);
            mat_x(&A, xn, kxn);
            round_f(kxn, m, o->fp32_bits & 2);
            for (int i = 0; i < m; ++i) {
                const double w = 2.0 * kxn[i] - kx[i] + y[i] / sigma;
                yn[i] = sigma * (w - clampd(w, rl[i], ru[i]));
                dy2 += (yn[i] - y[i]) * (yn[i] - y[i]);
            }
            round_f(yn, m, o->fp32_bits & 1);
            mat_ty(&A, yn, ktyn);
            round_f(ktyn, n, o->fp32_bits & 2);
            for (int j = 0; j < n; ++j) {
                const double dx = xn[j] - x[j];
                inter += dx * (ktyn[j] - kty[j]);
                dx2 += dx * dx;
            }
            const double movement = omega * dx2 + dy2 / omega;
            const double eta_bar = fabs(inter) > 0 ? movement / (2.0 * fabs(inter)) : INFINITY;
            /* PDLP counts iterations from 1: the base (k + 1) is at least 2 */
            const double k = (double)(attempts + 2);
            const double grow = (1.0 + pow(k, -0.6)) * eta;
            const double eta_next = isinf(eta_bar) ? grow : fmin((1.0 - pow(k, -0.3)) * eta_bar, grow);
            attempts++;
            if (eta <= eta_bar) {
                double* t;
                t = x; x = xn; xn = t;
                t = y; y = yn; yn = t;
                t = kx; kx = kxn; kxn = t;
                t = kty; kty = ktyn; ktyn = t;
                steps++;
                since++;
                W += eta;
                const double w = eta / W;
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
                for (int j = 0; j < n; ++j) x_avg[j] += w * (x[j] - x_avg[j]);
#pragma omp parallel for schedule(static) if (m > PAR_MIN)
                for (int i = 0; i < m; ++i) y_avg[i] += w * (y[i] - y_avg[i]);
                round_f(x_avg, n, o->fp32_bits & 4);
                round_f(y_avg, m, o->fp32_bits & 4);
            } else {
                rejections++;
            }
            eta = eta_next;
        }
    }
    free(xa_acc);
    free(ya_acc);
    const double* xs = out_sel ? x_avg : x;
    const double* ys = out_sel ? y_avg : y;
    for (int j = 0; j < n; ++j) x_out[j] = xs[j] * dcol[j];
    for (int i = 0; i < m; ++i) y_out[i] = ys[i] * drow[i];
    info->status = status;
    info->out_sel = out_sel;
    info->attempts = attempts;
    info->steps = steps;
    info->rejections = rejections;
    info->restarts = restarts;
    info->evals = evals;
    info->eta = eta;
    info->omega = omega;
    info->rel_p = ev[out_sel].rel_p;
    info->rel_d = ev[out_sel].rel_d;
    info->rel_g = ev[out_sel].rel_g;
    info->pobj = ev[out_sel].pobj;
    info->dobj = ev[out_sel].dobj;
    free(A.cp); free(A.ri); free(A.rp); free(A.ci); free(A.cv); free(A.rv);
    free(c); free(l); free(u); free(dcol); free(fc); free(rl); free(ru); free(drow); free(fr);
    free(x); free(xn); free(kty); free(ktyn); free(x_avg); free(x_last); free(kty_avg);
    free(y); free(yn); free(kx); free(kxn); free(y_avg); free(y_last); free(kx_avg);
    return 0;
}
