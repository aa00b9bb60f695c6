// Host-side problem preparation: validation of the C-ABI problem, FP64 -> FP32
// conversion into the engine's packed layout, and the FP64 KKT certificate.
#pragma once

#include <stdint.h>

#include <string>
#include <memory>
#include <utility>
#include <vector>

#include "sih_pdhg.h"

namespace sihg {

// One nonzero in the packed layout: {index, value}.  Same bytes as the int2
// {index, __float_as_int(value)} the kernels load.
struct Pair {
    int32_t idx;
    float val;
};

// Allocator whose resize leaves new elements default-initialised (no zero
// fill): the large entry arrays are written right after, by several threads.
template <class T>
struct NoInitAllocator : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInitAllocator<U>;
    };
    NoInitAllocator() = default;
    template <class U>
    NoInitAllocator(const NoInitAllocator<U>&) noexcept {}
    template <class U>
    void construct(U* p) noexcept {
        ::new ((void*)p) U;
    }
    template <class U, class... A>
    void construct(U* p, A&&... a) {
        ::new ((void*)p) U(std::forward<A>(a)...);
    }
};
using PairVec = std::vector<Pair, NoInitAllocator<Pair>>;

// The engine's host copy of one LP.
struct HostProblem {
    int m = 0, n = 0, nnz = 0;
    std::vector<int> csc_ptr;   // [n + 1]
    PairVec csc;                // [nnz] row index, value (columns' entries)
    std::vector<int> csr_ptr;   // [m + 1]
    PairVec csr;                // [nnz] column index, value (rows' entries, columns ascending)
    std::vector<float> c, l, u; // [n] FP32 casts (objective already multiplied by sense)
    std::vector<float> rl, ru;  // [m]
    const sih_pdhg_problem* src = nullptr; // original FP64 data (not owned)
    int sense = 1;
};

// Validates `p` and fills `hp` (multithreaded conversion).  Errors:
// SIH_PDHG_ERR_INVALID_ARGUMENT (with a message) or SIH_PDHG_ERR_UNSUPPORTED.
int build_host_problem(const sih_pdhg_problem* p, HostProblem& hp);

// Validation only (used by entry points before any device work).
int validate_problem(const sih_pdhg_problem* p);
int validate_config(const sih_pdhg_config* c);

struct KktReport {
    double rel_primal, rel_dual, rel_gap, primal_obj, dual_obj;
};

// FP64 KKT of (x, y_pdhg) for the ORIGINAL problem p (sense applied):
// primal residual of A x against the row bounds, dual residual of the reduced
// cost lambda = sense*c + A^T y that no finite bound can carry, duality gap;
// relative measures of docs/gpu_pdhg.md:51-57.  Optionally writes slack = A x
// and reduced_costs = sense * lambda (simplex convention, original sense).
KktReport host_kkt(const sih_pdhg_problem* p, const double* x, const double* y_pdhg, double* slack,
                   double* reduced_costs);

// Runs f(begin, end) over [0, count) split across hardware threads, at
// least `min_chunk` items per thread (parallel_for: 65,536).
template <class F>
void parallel_for_min(int64_t count, int64_t min_chunk, F&& f);
template <class F>
void parallel_for(int64_t count, F&& f) {
    parallel_for_min(count, (int64_t)1 << 16, static_cast<F&&>(f));
}

// Splits [0, count) into `parts` contiguous ranges (range t to part t) and runs
// f(begin, end, t) on them in parallel; below 2 x 65,536 items everything runs
// as part 0 on the calling thread.
template <class F>
void parallel_parts(int64_t count, int parts, F&& f);

bool bound_is_finite(double v);
int hardware_threads();

}  // namespace sihg

#include <thread>

namespace sihg {
template <class F>
void parallel_for_min(int64_t count, int64_t min_chunk, F&& f) {
    if (min_chunk < 1) min_chunk = 1;
    int t = hardware_threads();
    if (count < min_chunk * 2 || t <= 1) {
        f((int64_t)0, count);
        return;
    }
    int64_t chunks = (count + min_chunk - 1) / min_chunk;
    if (chunks < t) t = (int)chunks;
    std::vector<std::thread> pool;
    pool.reserve(t);
    for (int i = 0; i < t; ++i) {
        const int64_t b = count * i / t, e = count * (i + 1) / t;
        pool.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto& th : pool) th.join();
}

template <class F>
void parallel_parts(int64_t count, int parts, F&& f) {
    if (parts <= 1 || count < ((int64_t)1 << 17)) {
        f((int64_t)0, count, 0);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(parts);
    for (int t = 0; t < parts; ++t) {
        const int64_t b = count * t / parts, e = count * (t + 1) / parts;
        pool.emplace_back([&f, b, e, t] { f(b, e, t); });
    }
    for (auto& th : pool) th.join();
}
}  // namespace sihg
