// sih_pdhg_check_norms_noalloc: the reference's convergence measures without
// any allocation.
//
// Who needs it: callers that must not allocate device memory while they run,
// for example a host that gives every library a fixed device pool up front,
// or one that polls convergence from inside a loop where an allocation (and
// the implicit synchronisation of cudaMalloc / cudaFree) is not allowed.  Such
// a caller owns every input and output buffer; the working arrays the check
// needs come from a file-scope device array instead of cudaMalloc.
//
// What it computes (core/src/gpu/gpu_solver.cpp:242-259, with the reference's
// kernels core/src/gpu/cuda_pdhg.cu:14-49, 114-151): A x and A^T y, the
// per-row bound violation of A x and the per-column measure
// |x - clip(x - tau (c + A^T y), l, u)| / max(1e-4, tau), their maxima (NaN
// measures skipped, as the reference's host loop skips them), divided by
// max_abs_b and max_abs_c.  Same kernels and launch shapes as
// sih_pdhg_launch_csr_spmv / _csc_spmv / _residuals, so the two routes give
// the same bits.
#include <mutex>

#include "common.cuh"
#include "compat.cuh"

namespace sihg {

// Largest m + n the no-alloc check serves (524,288 rows plus columns): the
// array holds A x and A^T y (m + n floats), then the row violations and column
// measures (m + n floats), plus two reduction words.  Every GPU that loads the
// library keeps it (4 MiB + 256 bytes) until the process exits.
constexpr int kNoAllocMaxRowsCols = 1 << 19;
static __device__ __align__(256) float g_check_scratch[2 * kNoAllocMaxRowsCols + 64];

__global__ void noalloc_clear_kernel(unsigned* words) {
    if (threadIdx.x < 2) words[threadIdx.x] = 0u;
}

// Max of non-negative floats (NaN dropped by fmaxf) into words[which] (float bits).
__global__ void noalloc_max_kernel(int len, const float* __restrict__ v, unsigned* words, int which) {
    float mx = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) mx = fmaxf(mx, v[i]);
    __shared__ float red[32];
    mx = block_max_nonneg(mx, red);
    if (threadIdx.x == 0 && mx > 0.f) atomicMax(&words[which], __float_as_uint(mx));
}

__global__ void noalloc_finish_kernel(const unsigned* words, float max_abs_b, float max_abs_c, float* out) {
    if (threadIdx.x == 0) {
        out[0] = __uint_as_float(words[0]) / max_abs_b;
        out[1] = __uint_as_float(words[1]) / max_abs_c;
    }
}

static int lanes_for_mean(double mean) {  // the launchers' choice (compat.cu)
    int L = 1;
    while (L < 32 && 4.0 * L <= mean) L *= 2;
    return L;
}

static int grid_for(int n, int per_block, int sms) {
    return std::max(1, std::min((n + per_block - 1) / per_block, sms * 8));
}

// Id of the calling thread's current CUDA context (cuCtxGetId: unique for the
// life of the process, so a context re-created after cudaDeviceReset gets a
// new one).  The two driver calls are looked up through the runtime, so the
// library does not link the driver library itself.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

static int current_context_id(unsigned long long* id) {
    static std::once_flag once;
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    if (!get_current || !get_id) return fail(SIH_PDHG_ERR_CUDA, "driver entry points cuCtxGetCurrent / cuCtxGetId unavailable");
    void* ctx = nullptr;
    if (get_current(&ctx) != 0) return fail(SIH_PDHG_ERR_CUDA, "cuCtxGetCurrent failed");
    *id = 0;  // no context current yet: the runtime creates it at the first call that needs one
    if (ctx && get_id(ctx, id) != 0) return fail(SIH_PDHG_ERR_CUDA, "cuCtxGetId failed");
    return SIH_PDHG_OK;
}

// Device address of g_check_scratch (host code must not use the symbol itself
// as an address).  Set-up, with the device current: once per device, and again
// when the device's context is a new one (after cudaDeviceReset the module is
// loaded again and the array may sit elsewhere).  Later calls only compare the
// context id.
static int scratch_address(float** out, int* sms) {
    constexpr int kMaxDevices = 64;
    struct Entry {
        unsigned long long ctx_id = 0;
        float* addr = nullptr;
        int sm_count = 0;
    };
    static std::mutex mu;
    static Entry table[kMaxDevices];
    int dev = 0;
    SIHG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(SIH_PDHG_ERR_UNSUPPORTED, "device ordinal beyond 63");
    unsigned long long ctx_id = 0;
    SIHG_TRY(current_context_id(&ctx_id));
    std::lock_guard<std::mutex> g(mu);
    Entry& e = table[dev];
    if (!e.addr || ctx_id == 0 || e.ctx_id != ctx_id) {
        void* p = nullptr;
        SIHG_CUDA(cudaGetSymbolAddress(&p, g_check_scratch));  // makes the primary context current if none was
        if (ctx_id == 0) SIHG_TRY(current_context_id(&ctx_id));
        int s = 0;
        SIHG_CUDA(cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev));
        e.addr = static_cast<float*>(p);
        e.sm_count = s;
        e.ctx_id = ctx_id;
    }
    *out = e.addr;
    *sms = e.sm_count;
    return SIH_PDHG_OK;
}

static int check_norms_noalloc_impl(int m, int n, int nnz, const int* d_row_ptr, const int* d_col_ind,
                                    const float* d_csr_values, const int* d_col_ptr, const int* d_row_ind,
                                    const float* d_csc_values, const float* d_x, const float* d_y, const float* d_c,
                                    const float* d_l, const float* d_u, const float* d_tau, const float* d_row_l,
                                    const float* d_row_u, float max_abs_b, float max_abs_c, float* d_out,
                                    void* stream) {
    if (m < 1 || n < 1 || nnz < 0) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "m and n must be >= 1, nnz >= 0");
    if ((long long)m + (long long)n > kNoAllocMaxRowsCols)
        return fail(SIH_PDHG_ERR_INVALID_ARGUMENT,
                    "m + n = " + std::to_string((long long)m + n) + " exceeds the no-alloc limit of " +
                        std::to_string(kNoAllocMaxRowsCols) + " rows plus columns");
    if (!d_row_ptr || !d_col_ptr || !d_x || !d_y || !d_c || !d_l || !d_u || !d_tau || !d_row_l || !d_row_u || !d_out ||
        (nnz > 0 && (!d_col_ind || !d_csr_values || !d_row_ind || !d_csc_values)))
        return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    if (!(max_abs_b > 0.f) || !(max_abs_c > 0.f))
        return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "max_abs_b and max_abs_c must be > 0");
    float* scratch = nullptr;
    int sms = 1;
    SIHG_TRY(scratch_address(&scratch, &sms));
    float* ax = scratch;                                   // [m] A x
    float* aty = scratch + m;                              // [n] A^T y
    float* row_map = scratch + kNoAllocMaxRowsCols;        // [m] row violations
    float* col_map = row_map + m;                          // [n] column measures
    unsigned* words = reinterpret_cast<unsigned*>(scratch + 2 * kNoAllocMaxRowsCols);  // 2 max words
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    noalloc_clear_kernel<<<1, 32, 0, s>>>(words);
    const int Lr = lanes_for_mean((double)nnz / m), Lc = lanes_for_mean((double)nnz / n);
    split_spmv_kernel<<<grid_for(m, 256 / Lr, sms), 256, 0, s>>>(m, d_row_ptr, d_col_ind, d_csr_values, d_x, ax, Lr);
    split_spmv_kernel<<<grid_for(n, 256 / Lc, sms), 256, 0, s>>>(n, d_col_ptr, d_row_ind, d_csc_values, d_y, aty, Lc);
    compat_row_viol_kernel<<<grid_for(m, 256, sms), 256, 0, s>>>(m, ax, d_row_l, d_row_u, row_map);
    compat_col_viol_kernel<<<grid_for(n, 256, sms), 256, 0, s>>>(n, d_x, d_c, aty, d_l, d_u, d_tau, col_map);
    noalloc_max_kernel<<<grid_for(m, 256, sms), 256, 0, s>>>(m, row_map, words, 0);
    noalloc_max_kernel<<<grid_for(n, 256, sms), 256, 0, s>>>(n, col_map, words, 1);
    noalloc_finish_kernel<<<1, 32, 0, s>>>(words, max_abs_b, max_abs_c, d_out);
    SIHG_LAUNCH_CHECK();
    return SIH_PDHG_OK;
}

}  // namespace sihg

using namespace sihg;

extern "C" int sih_pdhg_check_norms_noalloc(int m, int n, int nnz, const int* d_row_ptr, const int* d_col_ind,
                                            const float* d_csr_values, const int* d_col_ptr, const int* d_row_ind,
                                            const float* d_csc_values, const float* d_x, const float* d_y,
                                            const float* d_c, const float* d_l, const float* d_u,
                                            const float* d_tau, const float* d_row_l, const float* d_row_u,
                                            float max_abs_b, float max_abs_c, float* d_out, void* stream) {
    return guarded([&] {
        return check_norms_noalloc_impl(m, n, nnz, d_row_ptr, d_col_ind, d_csr_values, d_col_ptr, d_row_ind,
                                        d_csc_values, d_x, d_y, d_c, d_l, d_u, d_tau, d_row_l, d_row_u, max_abs_b,
                                        max_abs_c, d_out, stream);
    });
}
