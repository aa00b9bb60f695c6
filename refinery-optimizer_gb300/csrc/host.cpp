// Host-side problem preparation and the FP64 KKT certificate.
#include "host.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <mutex>
#include <string>
#include <thread>

namespace sihg {

void set_last_error(const std::string& msg);

static int bad(const std::string& msg) {
    set_last_error(msg);
    return SIH_PDHG_ERR_INVALID_ARGUMENT;
}

int hardware_threads() {
    unsigned t = std::thread::hardware_concurrency();
    if (t == 0) t = 1;
    return (int)std::min(t, 32u);
}

// A bound counts as finite below 1e20 in magnitude (the reference's
// SIH_INF_THRESHOLD, core/include/sih/model/problem.hpp:27-35).
bool bound_is_finite(double v) { return !std::isinf(v) && std::fabs(v) < 1e20; }

int validate_config(const sih_pdhg_config* c) {
    if (!c) return bad("config is NULL");
    if (c->check_frequency <= 0) return bad("config.check_frequency must be > 0");
    if (c->max_iterations < 0) return bad("config.max_iterations must be >= 0");
    if (!(c->step_tau >= 0.0f) || !(c->step_sigma >= 0.0f)) return bad("config step sizes must be >= 0");
    return SIH_PDHG_OK;
}

int validate_problem(const sih_pdhg_problem* p) {
    if (!p) return bad("problem is NULL");
    if (p->num_rows < 0 || p->num_cols < 0 || p->num_nonzeros < 0) return bad("negative problem dimension");
    if (p->num_rows >= INT32_MAX || p->num_cols >= INT32_MAX || p->num_nonzeros >= INT32_MAX) {
        set_last_error("problem dimensions beyond 2^31-1 are not supported by the 32-bit index layout");
        return SIH_PDHG_ERR_UNSUPPORTED;
    }
    if (p->sense != 1 && p->sense != -1) return bad("sense must be 1 (minimize) or -1 (maximize)");
    const int64_t m = p->num_rows, n = p->num_cols, nnz = p->num_nonzeros;
    if (n > 0 && (!p->csc_col_ptr || !p->c || !p->col_lower || !p->col_upper))
        return bad("NULL column array (csc_col_ptr, c, col_lower or col_upper)");
    if (m > 0 && (!p->row_lower || !p->row_upper)) return bad("NULL row bound array");
    if (nnz > 0 && (!p->csc_row_ind || !p->csc_values)) return bad("NULL csc_row_ind or csc_values");
    const bool has_csr = p->csr_row_ptr || p->csr_col_ind || p->csr_values;
    if (has_csr && (!p->csr_row_ptr || (nnz > 0 && (!p->csr_col_ind || !p->csr_values))))
        return bad("CSR arrays must be all given or all NULL");
    if (n > 0) {
        if (p->csc_col_ptr[0] != 0 || p->csc_col_ptr[n] != nnz) return bad("csc_col_ptr must run from 0 to nnz");
        for (int64_t j = 0; j < n; ++j)
            if (p->csc_col_ptr[j + 1] < p->csc_col_ptr[j]) return bad("csc_col_ptr is not non-decreasing");
    } else if (nnz != 0) {
        return bad("nonzeros without columns");
    }
    if (has_csr && m > 0) {
        if (p->csr_row_ptr[0] != 0 || p->csr_row_ptr[m] != nnz) return bad("csr_row_ptr must run from 0 to nnz");
        for (int64_t i = 0; i < m; ++i)
            if (p->csr_row_ptr[i + 1] < p->csr_row_ptr[i]) return bad("csr_row_ptr is not non-decreasing");
    }
    for (int64_t i = 0; i < m; ++i)
        if (p->row_lower[i] > p->row_upper[i]) return bad("row_lower > row_upper at row " + std::to_string(i));
    for (int64_t j = 0; j < n; ++j)
        if (p->col_lower[j] > p->col_upper[j]) return bad("col_lower > col_upper at column " + std::to_string(j));
    return SIH_PDHG_OK;
}

int build_host_problem(const sih_pdhg_problem* p, HostProblem& hp) {
    int rc = validate_problem(p);
    if (rc != SIH_PDHG_OK) return rc;
    hp.src = p;
    hp.sense = p->sense;
    hp.m = (int)p->num_rows;
    hp.n = (int)p->num_cols;
    hp.nnz = (int)p->num_nonzeros;
    const int m = hp.m, n = hp.n, nnz = hp.nnz;
    hp.csc_ptr.resize((size_t)n + 1);
    hp.csc.resize((size_t)nnz);
    hp.c.resize(n);
    hp.l.resize(n);
    hp.u.resize(n);
    hp.rl.resize(m);
    hp.ru.resize(m);
    hp.csr_ptr.assign((size_t)m + 1, 0);
    // pointers and vectors in one pass: items [0, n] are columns (n: the last
    // pointer), items (n, n + 1 + m] rows
    parallel_for((int64_t)n + 1 + m + 1, [&](int64_t b, int64_t e) {
        for (int64_t k = b; k < e; ++k) {
            if (k <= n) {
                const int64_t j = k;
                hp.csc_ptr[j] = n > 0 ? (int)p->csc_col_ptr[j] : 0;
                if (j < n) {
                    hp.c[j] = (float)(p->sense == 1 ? p->c[j] : -p->c[j]);
                    hp.l[j] = (float)p->col_lower[j];
                    hp.u[j] = (float)p->col_upper[j];
                }
            } else {
                const int64_t i = k - n - 1;
                if (p->csr_row_ptr) hp.csr_ptr[i] = (int)p->csr_row_ptr[i];
                if (i < m) {
                    hp.rl[i] = (float)p->row_lower[i];
                    hp.ru[i] = (float)p->row_upper[i];
                }
            }
        }
    });
    // entries: the CSC, and the CSR when the problem brings one, in one pass
    // (items [0, nnz) CSC, [nnz, 2 nnz) CSR); every index is checked
    hp.csr.resize((size_t)nnz);
    std::atomic<int64_t> bad_csc{-1}, bad_csr{-1};
    const int64_t items = p->csr_row_ptr ? 2 * (int64_t)nnz : (int64_t)nnz;
    parallel_for(items, [&](int64_t b, int64_t e) {
        for (int64_t k = b; k < e; ++k) {
            if (k < nnz) {
                const int64_t r = p->csc_row_ind[k];
                if (r < 0 || r >= m) bad_csc.store(k);
                hp.csc[k] = Pair{(int32_t)r, (float)p->csc_values[k]};
            } else {
                const int64_t q = k - nnz, c = p->csr_col_ind[q];
                if (c < 0 || c >= n) bad_csr.store(q);
                hp.csr[q] = Pair{(int32_t)c, (float)p->csr_values[q]};
            }
        }
    });
    if (bad_csc.load() >= 0) return bad("csc_row_ind out of range at entry " + std::to_string(bad_csc.load()));
    if (bad_csr.load() >= 0) return bad("csr_col_ind out of range at entry " + std::to_string(bad_csr.load()));
    if (!p->csr_row_ptr) {
        // Counting-sort transpose in column order (columns ascending within a row),
        // the CSR the reference builds at core/src/gpu/gpu_solver.cpp:91-109.
        for (int k = 0; k < nnz; ++k) hp.csr_ptr[hp.csc[k].idx + 1]++;
        for (int i = 0; i < m; ++i) hp.csr_ptr[i + 1] += hp.csr_ptr[i];
        std::vector<int> fill(hp.csr_ptr.begin(), hp.csr_ptr.end() - 1);
        for (int j = 0; j < n; ++j)
            for (int k = hp.csc_ptr[j]; k < hp.csc_ptr[j + 1]; ++k) {
                const int r = hp.csc[k].idx;
                hp.csr[fill[r]++] = Pair{j, hp.csc[k].val};
            }
    }
    return SIH_PDHG_OK;
}

KktReport host_kkt(const sih_pdhg_problem* p, const double* x, const double* y, double* slack,
                   double* reduced_costs) {
    const int64_t m = p->num_rows, n = p->num_cols;
    const double sense = (double)p->sense;
    // A x: row by row from the problem's CSR, else one scatter pass over its CSC
    std::vector<double> ax;
    if (!p->csr_row_ptr) {
        ax.assign((size_t)m, 0.0);
        for (int64_t j = 0; j < n; ++j)
            for (int64_t k = p->csc_col_ptr[j]; k < p->csc_col_ptr[j + 1]; ++k)
                ax[p->csc_row_ind[k]] += p->csc_values[k] * x[j];
    }
    // per-thread partials, combined in thread order (a fixed split per thread count)
    struct Part {
        double pobj = 0, dobj = 0, rd = 0, cinf = 0, rp = 0, binf = 0;
    };
    const int T = std::max(1, hardware_threads());
    std::vector<Part> rows(T), cols(T);
    auto row_work = [&](int64_t b, int64_t e, int t) {
        Part& P = rows[t];
        for (int64_t i = b; i < e; ++i) {
            double a;
            if (p->csr_row_ptr) {
                a = 0.0;
                for (int64_t k = p->csr_row_ptr[i]; k < p->csr_row_ptr[i + 1]; ++k)
                    a += p->csr_values[k] * x[p->csr_col_ind[k]];
            } else {
                a = ax[i];
            }
            const double lo = p->row_lower[i], hi = p->row_upper[i];
            double r = 0.0;
            if (bound_is_finite(lo)) { P.binf = std::max(P.binf, std::fabs(lo)); if (a < lo) r = lo - a; }
            if (bound_is_finite(hi)) { P.binf = std::max(P.binf, std::fabs(hi)); if (a > hi) r = a - hi; }
            P.rp = std::max(P.rp, r);
            const double yn = y[i] < 0 ? -y[i] : 0.0, yp = y[i] > 0 ? y[i] : 0.0;
            if (bound_is_finite(lo)) P.dobj += yn * lo; else P.rd = std::max(P.rd, yn);
            if (bound_is_finite(hi)) P.dobj -= yp * hi; else P.rd = std::max(P.rd, yp);
            if (slack) slack[i] = a;
        }
    };
    auto col_work = [&](int64_t b, int64_t e, int t) {
        Part& P = cols[t];
        for (int64_t j = b; j < e; ++j) {
            const double cj = sense * p->c[j];
            double lam = cj;
            for (int64_t k = p->csc_col_ptr[j]; k < p->csc_col_ptr[j + 1]; ++k)
                lam += p->csc_values[k] * y[p->csc_row_ind[k]];
            if (reduced_costs) reduced_costs[j] = sense * lam;
            P.pobj += cj * x[j];
            P.cinf = std::max(P.cinf, std::fabs(cj));
            const double pos = lam > 0 ? lam : 0.0, neg = lam < 0 ? -lam : 0.0;
            if (bound_is_finite(p->col_lower[j])) P.dobj += pos * p->col_lower[j]; else P.rd = std::max(P.rd, pos);
            if (bound_is_finite(p->col_upper[j])) P.dobj -= neg * p->col_upper[j]; else P.rd = std::max(P.rd, neg);
        }
    };
    parallel_parts(n, T, col_work);
    parallel_parts(m, T, row_work);
    double pobj = 0, dobj = 0, rd_inf = 0, c_inf = 0, rp_inf = 0, b_inf = 0;
    for (int t = 0; t < T; ++t) {
        pobj += cols[t].pobj;
        dobj += cols[t].dobj;
        rd_inf = std::max(rd_inf, cols[t].rd);
        c_inf = std::max(c_inf, cols[t].cinf);
    }
    for (int t = 0; t < T; ++t) {
        dobj += rows[t].dobj;
        rd_inf = std::max(rd_inf, rows[t].rd);
        rp_inf = std::max(rp_inf, rows[t].rp);
        b_inf = std::max(b_inf, rows[t].binf);
    }
    KktReport r;
    r.rel_primal = rp_inf / (1.0 + b_inf);
    r.rel_dual = rd_inf / (1.0 + c_inf);
    r.rel_gap = std::fabs(pobj - dobj) / (1.0 + std::fabs(pobj) + std::fabs(dobj));
    r.primal_obj = pobj;
    r.dual_obj = dobj;
    return r;
}

}  // namespace sihg
