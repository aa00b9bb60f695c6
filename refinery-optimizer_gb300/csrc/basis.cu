// Basis guess of the hybrid polish on the device (sih_pdhg_basis_guess).
//
// The reference's GpuSolver::solve_hybrid (core/src/gpu/gpu_solver.cpp:332-395)
// scores every column (its value x_j) and every row (its activity (A x)_i) by
// the distance to its nearer finite bound (a bound beyond +-1e15 counts as
// absent, distance 1e30), sorts the n + m candidates by descending distance
// on the host and makes the first m basic; the others sit at their nearer
// bound (at lower when the distances tie).  Here the scoring and the top-m
// selection run on the GPU:
//   1. k_score: distance (FP64, the reference's formula) -> 64-bit key (the
//      bits of a non-negative double order like the value) and the side flag;
//   2. radix select, most significant byte first: per pass a histogram of the
//      next byte of the keys that match the selected prefix (k_hist), then one
//      thread picks the byte whose bucket holds the m-th largest key
//      (k_select_step); after eight passes the m-th largest key T is known and
//      how many of the keys equal to T are still to take;
//   3. k_tie_count / k_tie_scan / k_mark: keys above T are basic; of the keys
//      equal to T the ones with the lowest candidate index are taken (blocks
//      own contiguous index ranges; a block-count scan gives each block its
//      offset), which is the order a stable descending sort gives ties.
// Candidates are columns 0..n-1 then rows n..n+m-1, as in the reference.
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "host.h"

namespace sihg {
namespace {

constexpr int kBasisThreads = 256;

struct SelectState {
    unsigned long long prefix;  // selected high bytes of T
    unsigned long long mask;    // bits of the prefix fixed so far
    long long need;             // keys still to take among those matching the prefix
    long long above;            // keys above the prefix (all basic)
};

__device__ __forceinline__ double bound_distance(double v, double lo, double hi, bool& at_lower) {
    const double dl = lo > -1e15 ? fmax(0.0, v - lo) : 1e30;
    const double du = hi < 1e15 ? fmax(0.0, hi - v) : 1e30;
    at_lower = dl <= du;
    return fmin(dl, du);
}

__global__ void k_score(long long n, long long m, const double* __restrict__ x, const double* __restrict__ ax,
                        const double* __restrict__ cl, const double* __restrict__ cu, const double* __restrict__ rl,
                        const double* __restrict__ ru, unsigned long long* __restrict__ key,
                        unsigned char* __restrict__ lower) {
    const long long K = n + m;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < K; t += (long long)gridDim.x * blockDim.x) {
        bool at_lower;
        const double d = t < n ? bound_distance(x[t], cl[t], cu[t], at_lower)
                               : bound_distance(ax[t - n], rl[t - n], ru[t - n], at_lower);
        // d >= 0: the bits order like the value (a zero distance is +0, so -0 and +0 tie as in the host sort)
        key[t] = d == 0.0 ? 0ull : (unsigned long long)__double_as_longlong(d);
        lower[t] = at_lower ? 1 : 0;
    }
}

__global__ void k_hist(long long K, const unsigned long long* __restrict__ key, const SelectState* __restrict__ st,
                       int shift, unsigned* __restrict__ hist) {
    __shared__ unsigned h[256];
    for (int b = threadIdx.x; b < 256; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const unsigned long long prefix = st->prefix, mask = st->mask;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < K; t += (long long)gridDim.x * blockDim.x) {
        const unsigned long long k = key[t];
        if ((k & mask) == prefix) atomicAdd(&h[(k >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 256; b += blockDim.x)
        if (h[b]) atomicAdd(&hist[b], h[b]);
}

// One thread: the byte at `shift` of the m-th largest key; zeroes the histogram
// for the next pass.
__global__ void k_select_step(SelectState* st, int shift, unsigned* hist) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    SelectState s = *st;
    long long need = s.need;
    int pick = 0;
    for (int b = 255; b >= 0; --b) {
        const long long c = hist[b];
        if (c >= need) {
            pick = b;
            break;
        }
        need -= c;
        s.above += c;
    }
    s.prefix |= (unsigned long long)pick << shift;
    s.mask |= 0xffull << shift;
    s.need = need;
    *st = s;
    for (int b = 0; b < 256; ++b) hist[b] = 0;
}

// Keys equal to T per block range [blk * chunk, (blk + 1) * chunk).
__global__ void k_tie_count(long long K, long long chunk, const unsigned long long* __restrict__ key,
                            const SelectState* __restrict__ st, unsigned long long* __restrict__ counts) {
    __shared__ unsigned long long sum;
    if (threadIdx.x == 0) sum = 0;
    __syncthreads();
    const unsigned long long T = st->prefix;
    const long long b0 = blockIdx.x * chunk, b1 = min(K, b0 + chunk);
    unsigned long long c = 0;
    for (long long t = b0 + threadIdx.x; t < b1; t += blockDim.x) c += key[t] == T;
    atomicAdd(&sum, c);
    __syncthreads();
    if (threadIdx.x == 0) counts[blockIdx.x] = sum;
}

// Exclusive prefix of the block counts (one thread; the grid is small).
__global__ void k_tie_scan(int nb, unsigned long long* counts) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long acc = 0;
    for (int b = 0; b < nb; ++b) {
        const unsigned long long c = counts[b];
        counts[b] = acc;
        acc += c;
    }
}

// Status of every candidate: 0 basic, 1 at lower, 2 at upper (the values of
// sih::model::BasisStatus, core/include/sih/model/solution.hpp:23-29).
__global__ void k_mark(long long K, long long chunk, const unsigned long long* __restrict__ key,
                       const unsigned char* __restrict__ lower, const SelectState* __restrict__ st,
                       const unsigned long long* __restrict__ offsets, signed char* __restrict__ status) {
    __shared__ unsigned long long warp_tot[kBasisThreads / 32];
    __shared__ unsigned long long run;
    const unsigned long long T = st->prefix;
    const long long need = st->need;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) run = offsets[blockIdx.x];
    __syncthreads();
    const long long b0 = blockIdx.x * chunk, b1 = min(K, b0 + chunk);
    for (long long base = b0; base < b1; base += blockDim.x) {
        const long long t = base + threadIdx.x;
        const bool in = t < b1;
        const unsigned long long k = in ? key[t] : 0ull;
        const bool tie = in && k == T;
        // rank of this tie among the ties of lower index
        const unsigned bal = __ballot_sync(FULL_MASK, tie);
        const unsigned before_in_warp = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) warp_tot[warp] = __popc(bal);
        __syncthreads();
        unsigned long long before = run + before_in_warp;
        for (int w = 0; w < warp; ++w) before += warp_tot[w];
        if (in) {
            const bool basic = k > T || (tie && (long long)before < need);
            status[t] = basic ? 0 : (lower[t] ? 1 : 2);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long s = 0;
            for (int w = 0; w < kBasisThreads / 32; ++w) s += warp_tot[w];
            run += s;
        }
        __syncthreads();
    }
}

int basis_guess_impl(const sih_pdhg_problem* p, const double* x, const double* row_activity, int8_t* col_status,
                     int8_t* row_status) {
    if (!p || !x || (!row_activity && p->num_rows > 0) || !col_status || (!row_status && p->num_rows > 0))
        return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "basis guess: NULL argument");
    const long long n = p->num_cols, m = p->num_rows, K = n + m;
    if (n < 0 || m < 0) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "basis guess: negative size");
    if (!p->col_lower || !p->col_upper || (m > 0 && (!p->row_lower || !p->row_upper)))
        return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "basis guess: NULL bound array");
    if (K == 0) return SIH_PDHG_OK;
    int dev = 0, sms = 1;
    SIHG_CUDA(cudaGetDevice(&dev));
    SIHG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s = nullptr;
    SIHG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{s};
    // device buffers: x, activity, four bound arrays (FP64), keys, side flags, status
    DevMem dbl, keys, flags, stat, sel, hist, counts;
    const size_t nd = (size_t)K * 3;  // values, lowers, uppers (columns then rows)
    SIHG_TRY(dbl.alloc(sizeof(double) * nd));
    double* dv = dbl.as<double>();
    double* dlo = dv + K;
    double* dhi = dlo + K;
    SIHG_CUDA(cudaMemcpyAsync(dv, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(dlo, p->col_lower, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemcpyAsync(dhi, p->col_upper, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    if (m > 0) {
        SIHG_CUDA(cudaMemcpyAsync(dv + n, row_activity, sizeof(double) * m, cudaMemcpyHostToDevice, s));
        SIHG_CUDA(cudaMemcpyAsync(dlo + n, p->row_lower, sizeof(double) * m, cudaMemcpyHostToDevice, s));
        SIHG_CUDA(cudaMemcpyAsync(dhi + n, p->row_upper, sizeof(double) * m, cudaMemcpyHostToDevice, s));
    }
    SIHG_TRY(keys.alloc(sizeof(unsigned long long) * K));
    SIHG_TRY(flags.alloc((size_t)K));
    SIHG_TRY(stat.alloc((size_t)K));
    SIHG_TRY(sel.alloc(sizeof(SelectState)));
    SIHG_TRY(hist.alloc(sizeof(unsigned) * 256));
    const int grid = (int)std::max<long long>(1, std::min<long long>(sms * 8LL, (K + kBasisThreads - 1) / kBasisThreads));
    k_score<<<grid, kBasisThreads, 0, s>>>(n, m, dv, dv + n, dlo, dhi, dlo + n, dhi + n,
                                           keys.as<unsigned long long>(), flags.as<unsigned char>());
    const SelectState init{0ull, 0ull, m, 0};
    SIHG_CUDA(cudaMemcpyAsync(sel.as<void>(), &init, sizeof(init), cudaMemcpyHostToDevice, s));
    SIHG_CUDA(cudaMemsetAsync(hist.as<void>(), 0, sizeof(unsigned) * 256, s));
    if (m > 0) {
        for (int shift = 56; shift >= 0; shift -= 8) {
            k_hist<<<grid, kBasisThreads, 0, s>>>(K, keys.as<unsigned long long>(), sel.as<SelectState>(), shift,
                                                  hist.as<unsigned>());
            k_select_step<<<1, 32, 0, s>>>(sel.as<SelectState>(), shift, hist.as<unsigned>());
        }
    } else {  // no row: nothing is basic (T above every key)
        const SelectState none{~0ull, ~0ull, 0, 0};
        SIHG_CUDA(cudaMemcpyAsync(sel.as<void>(), &none, sizeof(none), cudaMemcpyHostToDevice, s));
    }
    const long long chunk = std::max<long long>(kBasisThreads, (K + grid - 1) / grid);
    const int nb = (int)((K + chunk - 1) / chunk);
    SIHG_TRY(counts.alloc(sizeof(unsigned long long) * nb));
    k_tie_count<<<nb, kBasisThreads, 0, s>>>(K, chunk, keys.as<unsigned long long>(), sel.as<SelectState>(),
                                             counts.as<unsigned long long>());
    k_tie_scan<<<1, 32, 0, s>>>(nb, counts.as<unsigned long long>());
    k_mark<<<nb, kBasisThreads, 0, s>>>(K, chunk, keys.as<unsigned long long>(), flags.as<unsigned char>(),
                                        sel.as<SelectState>(), counts.as<unsigned long long>(), stat.as<signed char>());
    SIHG_LAUNCH_CHECK();
    SIHG_CUDA(cudaMemcpyAsync(col_status, stat.as<signed char>(), (size_t)n, cudaMemcpyDeviceToHost, s));
    if (m > 0) SIHG_CUDA(cudaMemcpyAsync(row_status, stat.as<signed char>() + n, (size_t)m, cudaMemcpyDeviceToHost, s));
    SIHG_CUDA(cudaStreamSynchronize(s));
    return SIH_PDHG_OK;
}

}  // namespace

bool device_present();

}  // namespace sihg

extern "C" int sih_pdhg_basis_guess(const sih_pdhg_problem* problem, const double* x, const double* row_activity,
                                    int8_t* col_status, int8_t* row_status) {
    using namespace sihg;
    return guarded([&]() -> int {
        if (!device_present()) return fail(SIH_PDHG_ERR_NO_DEVICE, "no CUDA device (this engine has no CPU fallback)");
        return basis_guess_impl(problem, x, row_activity, col_status, row_status);
    });
}
