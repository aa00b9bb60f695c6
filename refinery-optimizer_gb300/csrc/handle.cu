// Handle API: problems stay resident on the device between solves.
#include <memory>
#include <vector>

#include "common.cuh"
#include "host.h"
#include "mixed.h"
#include "plain.h"

using namespace sihg;

struct sih_pdhg_handle {
    sih_pdhg_config cfg{};
    sih_pdhg_options opts{};
    std::vector<HostProblem> hps;
    std::unique_ptr<MixedSolver> mixed;
    std::vector<std::unique_ptr<PlainSolver>> plain;
    bool ran = false;
};

namespace sihg {
int solve_plain_packed(PlainSolver& solver, const HostProblem& hp, const sih_pdhg_options& opts, sih_pdhg_result* r);
void clear_result_scalars(sih_pdhg_result* r);
int resolve_options(const sih_pdhg_options* in, sih_pdhg_options& out);
bool device_present();

// Bytes the upload of one instance moves host -> device: packed CSR and CSC
// pairs, both pointer arrays and the five data vectors.
uint64_t instance_h2d_bytes(const HostProblem& p) {
    return 16ull * p.nnz + 4ull * (p.m + 1) + 4ull * (p.n + 1) + 4ull * (3ull * p.n + 2ull * p.m);
}

// The mixed path also uploads, per segment, its source entry and instance
// offset (int2) and the inverse of the renumbering (int).
uint64_t mixed_h2d_bytes(const HostProblem& p) { return instance_h2d_bytes(p) + 12ull * ((uint64_t)p.n + p.m); }
}  // namespace sihg

extern "C" {

static int create_impl(const sih_pdhg_problem* problems, int32_t count, const sih_pdhg_config* config,
                    const sih_pdhg_options* opts_in, sih_pdhg_handle** out) {
    if (!out) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!problems || count < 1) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "need at least one problem");
    SIHG_TRY(validate_config(config));
    auto h = std::make_unique<sih_pdhg_handle>();
    h->cfg = *config;
    SIHG_TRY(resolve_options(opts_in, h->opts));
    h->hps.resize(count);
    for (int b = 0; b < count; ++b) {
        int rc = build_host_problem(&problems[b], h->hps[b]);
        if (rc != SIH_PDHG_OK) {
            set_last_error("problem " + std::to_string(b) + ": " + std::string(sih_pdhg_last_error()));
            return rc;
        }
        if (h->hps[b].m == 0 || h->hps[b].n == 0)
            return fail(SIH_PDHG_ERR_UNSUPPORTED, "empty instances are not supported by the handle API");
    }
    if (!device_present()) return fail(SIH_PDHG_ERR_NO_DEVICE, "no CUDA device (this engine has no CPU fallback)");
    if (h->opts.algorithm == SIH_PDHG_ALGO_MIXED) {
        std::vector<const HostProblem*> ptrs;
        for (auto& p : h->hps) ptrs.push_back(&p);
        h->mixed = std::make_unique<MixedSolver>();
        SIHG_TRY(h->mixed->setup(ptrs, h->cfg, h->opts));
    } else {
        for (auto& p : h->hps) {
            h->plain.push_back(std::make_unique<PlainSolver>());
            SIHG_TRY(h->plain.back()->setup(p, h->cfg, h->opts));
        }
    }
    *out = h.release();
    return SIH_PDHG_OK;
}

int sih_pdhg_create(const sih_pdhg_problem* problems, int32_t count, const sih_pdhg_config* config,
                    const sih_pdhg_options* opts_in, sih_pdhg_handle** out) {
    return guarded([&] { return create_impl(problems, count, config, opts_in, out); });
}

static int run_impl(sih_pdhg_handle* h, double* device_seconds) {
    if (!h) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "handle is NULL");
    double secs = 0.0;
    if (h->mixed) {
        SIHG_TRY(h->mixed->run());
        secs = h->mixed->loop_seconds();
    } else {
        for (auto& s : h->plain) {
            SIHG_TRY(s->iterate());
            secs += s->loop_seconds();
        }
    }
    h->ran = true;
    if (device_seconds) *device_seconds = secs;
    return SIH_PDHG_OK;
}

int sih_pdhg_run(sih_pdhg_handle* h, double* device_seconds) {
    return guarded([&] { return run_impl(h, device_seconds); });
}

static int get_result_impl(sih_pdhg_handle* h, int32_t index, sih_pdhg_result* r) {
    if (!h || !r) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "NULL handle or result");
    if (index < 0 || index >= (int32_t)h->hps.size()) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "index out of range");
    if (!h->ran) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "sih_pdhg_run has not been called");
    clear_result_scalars(r);
    const HostProblem& hp = h->hps[index];
    if (h->mixed) {
        std::vector<double> x, y;
        SIHG_TRY(h->mixed->fetch(index, x, y));
        h->mixed->fill_result(index, r);
        pack_solution(hp.src, h->opts, x, y, r);
        r->d2h_bytes = 8ull * (hp.n + hp.m);
    } else {
        SIHG_TRY(solve_plain_packed(*h->plain[index], hp, h->opts, r));
    }
    r->h2d_bytes = h->mixed ? mixed_h2d_bytes(hp) : instance_h2d_bytes(hp);
    return SIH_PDHG_OK;
}

int sih_pdhg_get_result(sih_pdhg_handle* h, int32_t index, sih_pdhg_result* r) {
    return guarded([&] { return get_result_impl(h, index, r); });
}

static int time_kernels_impl(sih_pdhg_handle* h, int32_t reps, double* seconds, double* bytes) {
    if (!h || !seconds || reps < 1) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "bad arguments");
    if (!h->mixed) return fail(SIH_PDHG_ERR_UNSUPPORTED, "kernel timing is available for the mixed algorithm");
    return h->mixed->time_kernels(reps, seconds, bytes);
}

int sih_pdhg_time_kernels(sih_pdhg_handle* h, int32_t reps, double* seconds, double* bytes) {
    return guarded([&] { return time_kernels_impl(h, reps, seconds, bytes); });
}

static int set_start_impl(sih_pdhg_handle* h, int32_t index, const double* x, const double* row_duals,
                       double primal_weight) {
    if (!h) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "NULL handle");
    if (!h->mixed) return fail(SIH_PDHG_ERR_UNSUPPORTED, "warm starts are available for the mixed algorithm");
    return h->mixed->set_start(index, x, row_duals, primal_weight);
}

int sih_pdhg_set_start(sih_pdhg_handle* h, int32_t index, const double* x, const double* row_duals,
                       double primal_weight) {
    return guarded([&] { return set_start_impl(h, index, x, row_duals, primal_weight); });
}

int sih_pdhg_get_task_nnz(const sih_pdhg_handle* h, int32_t* task_nnz) {
    if (!h || !task_nnz) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!h->mixed) return fail(SIH_PDHG_ERR_UNSUPPORTED, "task sizes belong to the mixed algorithm");
    *task_nnz = h->mixed->task_nnz();
    return SIH_PDHG_OK;
}

int sih_pdhg_get_launch_shape(const sih_pdhg_handle* h, sih_pdhg_launch_shape* shape) {
    if (!h || !shape) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!h->mixed) return fail(SIH_PDHG_ERR_UNSUPPORTED, "launch shapes belong to the mixed algorithm");
    h->mixed->launch_shape(shape);
    return SIH_PDHG_OK;
}

void sih_pdhg_destroy(sih_pdhg_handle* h) { delete h; }

int sih_pdhg_check_grid_barrier(int32_t blocks, int32_t missing, int32_t rounds, double limit_sec,
                                int32_t* timed_out, int32_t* passed) {
    return guarded([&]() -> int {
        if (!device_present()) return fail(SIH_PDHG_ERR_NO_DEVICE, "no CUDA device");
        int t = 0, p = 0;
        SIHG_TRY(check_grid_barrier(blocks, missing, rounds, limit_sec, &t, &p));
        if (timed_out) *timed_out = t;
        if (passed) *passed = p;
        return SIH_PDHG_OK;
    });
}

static int solve_batch_impl(const sih_pdhg_problem* problems, int32_t count, const sih_pdhg_config* config,
                         const sih_pdhg_options* opts, sih_pdhg_result* results) {
    if (!results) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "results is NULL");
    sih_pdhg_handle* h = nullptr;
    SIHG_TRY(sih_pdhg_create(problems, count, config, opts, &h));
    std::unique_ptr<sih_pdhg_handle> guard(h);
    double secs = 0.0;
    SIHG_TRY(sih_pdhg_run(h, &secs));
    for (int b = 0; b < count; ++b) {
        SIHG_TRY(sih_pdhg_get_result(h, b, &results[b]));
        results[b].time_solver_sec = secs;
    }
    return SIH_PDHG_OK;
}

int sih_pdhg_solve_batch(const sih_pdhg_problem* problems, int32_t count, const sih_pdhg_config* config,
                         const sih_pdhg_options* opts, sih_pdhg_result* results) {
    return guarded([&] { return solve_batch_impl(problems, count, config, opts, results); });
}

}  // extern "C"
