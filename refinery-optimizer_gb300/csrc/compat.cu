// The reference's kernel launchers (core/src/gpu/cuda_pdhg.cu:155-203) with
// their exact argument lists: separate int32 index and float value arrays,
// device pointers, a caller stream.  The reference's host driver binds them at
// core/src/gpu/gpu_solver.cpp:18-40.  The SpMVs use warp-cooperative segment
// groups (lanes chosen from the mean segment length); updates are the
// reference's element formulas with unfused float operations.
#include <algorithm>
#include <map>
#include <mutex>

#include "common.cuh"

namespace sihg {

__device__ __forceinline__ float split_dot(const int* __restrict__ idx, const float* __restrict__ val, int beg,
                                           int end, int lane0, int L, const float* __restrict__ vec) {
    float s0 = 0.f, s1 = 0.f;
    int k = beg + lane0;
    for (; k + L < end; k += 2 * L) {
        s0 = fmaf(__ldg(val + k), __ldg(vec + __ldg(idx + k)), s0);
        s1 = fmaf(__ldg(val + k + L), __ldg(vec + __ldg(idx + k + L)), s1);
    }
    if (k < end) s0 = fmaf(__ldg(val + k), __ldg(vec + __ldg(idx + k)), s0);
    return s0 + s1;
}

__global__ void __launch_bounds__(256) split_spmv_kernel(int nseg, const int* __restrict__ ptr,
                                                         const int* __restrict__ idx,
                                                         const float* __restrict__ val,
                                                         const float* __restrict__ vec, float* __restrict__ out,
                                                         int L) {
    const int lane = threadIdx.x & 31, sub = lane & (L - 1), gpw = 32 / L;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int base = wid * gpw; base < nseg; base += nw * gpw) {
        const int r = base + lane / L;
        float s = 0.f;
        if (r < nseg) s = split_dot(idx, val, ptr[r], ptr[r + 1], sub, L, vec);
        for (int o = L >> 1; o > 0; o >>= 1) s += __shfl_down_sync(FULL_MASK, s, o, L);
        if (r < nseg && sub == 0) out[r] = s;
    }
}

__global__ void compat_primal_kernel(int n, const float* __restrict__ tau, const float* __restrict__ c,
                                     const float* __restrict__ aty, const float* __restrict__ l,
                                     const float* __restrict__ u, float* __restrict__ x,
                                     float* __restrict__ xbar) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const float x_old = x[j];
        float x_new = __fsub_rn(x_old, __fmul_rn(tau[j], __fadd_rn(c[j], aty[j])));
        if (x_new < l[j]) x_new = l[j];
        if (x_new > u[j]) x_new = u[j];
        x[j] = x_new;
        xbar[j] = __fsub_rn(__fmul_rn(2.0f, x_new), x_old);
    }
}

__global__ void compat_dual_kernel(int m, const float* __restrict__ sigma, const float* __restrict__ axbar,
                                   const float* __restrict__ rl, const float* __restrict__ ru,
                                   float* __restrict__ y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const float sig = sigma[i];
        const float w = __fadd_rn(axbar[i], y[i] / sig);
        float p = w;
        if (p < rl[i]) p = rl[i];
        if (p > ru[i]) p = ru[i];
        y[i] = __fmul_rn(sig, __fsub_rn(w, p));
    }
}

__global__ void compat_copy_kernel(int n, const float* __restrict__ x, float* __restrict__ xbar) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) xbar[j] = x[j];
}

__global__ void compat_row_viol_kernel(int m, const float* __restrict__ ax, const float* __restrict__ rl,
                                       const float* __restrict__ ru, float* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const float a = ax[i];
        float viol = 0.0f;
        if (rl[i] > -1e15f && a < rl[i]) viol = fmaxf(viol, __fsub_rn(rl[i], a));
        if (ru[i] < 1e15f && a > ru[i]) viol = fmaxf(viol, __fsub_rn(a, ru[i]));
        out[i] = viol;
    }
}

__global__ void compat_col_viol_kernel(int n, const float* __restrict__ x, const float* __restrict__ c,
                                       const float* __restrict__ aty, const float* __restrict__ l,
                                       const float* __restrict__ u, const float* __restrict__ tau,
                                       float* __restrict__ out) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const float xj = x[j], step = tau[j];
        float proj = __fsub_rn(xj, __fmul_rn(step, __fadd_rn(c[j], aty[j])));
        if (proj < l[j]) proj = l[j];
        if (proj > u[j]) proj = u[j];
        out[j] = fabsf(__fsub_rn(xj, proj)) / fmaxf(1e-4f, step);
    }
}

static int grid_for(int n, int per_block) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return std::max(1, std::min((n + per_block - 1) / per_block, sms * 8));
}

// Lanes per segment from the mean segment length.  The last pointer is read
// once per (pointer, size) and cached, so only the first launch on a matrix
// synchronizes its stream.
static int lanes_for(int nseg, const int* d_ptr, cudaStream_t s) {
    static std::mutex mu;
    static std::map<std::pair<const int*, int>, int> cache;
    {
        std::lock_guard<std::mutex> g(mu);
        auto it = cache.find({d_ptr, nseg});
        if (it != cache.end()) return it->second;
    }
    int nnz = 0;
    if (nseg > 0) {
        cudaMemcpyAsync(&nnz, d_ptr + nseg, sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
    }
    const double mean = nseg > 0 ? (double)nnz / nseg : 1.0;
    int L = 1;
    while (L < 32 && 4.0 * L <= mean) L *= 2;
    std::lock_guard<std::mutex> g(mu);
    cache[{d_ptr, nseg}] = L;
    return L;
}

static int split_spmv(int nseg, const int* ptr, const int* idx, const float* val, const float* vec, float* out,
                      void* stream) {
    if (nseg < 0) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "negative dimension");
    if (nseg == 0) return SIH_PDHG_OK;
    if (!ptr || !out || !vec) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "NULL device pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int L = lanes_for(nseg, ptr, s);
    split_spmv_kernel<<<grid_for(nseg, 256 / L), 256, 0, s>>>(nseg, ptr, idx, val, vec, out, L);
    SIHG_LAUNCH_CHECK();
    return SIH_PDHG_OK;
}

}  // namespace sihg

using namespace sihg;

// Every launcher runs inside guarded(): the lane cache (std::map, std::mutex)
// and the error messages can throw, and no exception may cross the C ABI.
extern "C" int sih_pdhg_launch_csr_spmv(int m, const int* d_row_ptr, const int* d_col_ind, const float* d_values,
                                        const float* d_x, float* d_y, void* stream) {
    return guarded([&] { return split_spmv(m, d_row_ptr, d_col_ind, d_values, d_x, d_y, stream); });
}

extern "C" int sih_pdhg_launch_csc_spmv(int n, const int* d_col_ptr, const int* d_row_ind, const float* d_values,
                                        const float* d_y, float* d_z, void* stream) {
    return guarded([&] { return split_spmv(n, d_col_ptr, d_row_ind, d_values, d_y, d_z, stream); });
}

extern "C" int sih_pdhg_launch_primal_update(int n, const float* d_tau, const float* d_c, const float* d_AT_y,
                                             const float* d_l, const float* d_u, float* d_x, float* d_x_bar,
                                             void* stream) {
    return guarded([&]() -> int {
        if (n < 0) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "negative dimension");
        if (n == 0) return SIH_PDHG_OK;
        compat_primal_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, d_tau, d_c, d_AT_y, d_l, d_u, d_x,
                                                                                 d_x_bar);
        SIHG_LAUNCH_CHECK();
        return SIH_PDHG_OK;
    });
}

extern "C" int sih_pdhg_launch_dual_update(int m, const float* d_sigma, const float* d_A_xbar, const float* d_row_l,
                                           const float* d_row_u, float* d_y, void* stream) {
    return guarded([&]() -> int {
        if (m < 0) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "negative dimension");
        if (m == 0) return SIH_PDHG_OK;
        compat_dual_kernel<<<grid_for(m, 256), 256, 0, (cudaStream_t)stream>>>(m, d_sigma, d_A_xbar, d_row_l, d_row_u,
                                                                               d_y);
        SIHG_LAUNCH_CHECK();
        return SIH_PDHG_OK;
    });
}

extern "C" int sih_pdhg_launch_restart(int n, const float* d_x, float* d_x_bar, void* stream) {
    return guarded([&]() -> int {
        if (n < 0) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "negative dimension");
        if (n == 0) return SIH_PDHG_OK;
        compat_copy_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, d_x, d_x_bar);
        SIHG_LAUNCH_CHECK();
        return SIH_PDHG_OK;
    });
}

extern "C" int sih_pdhg_launch_residuals(int m, int n, const float* d_Ax, const float* d_row_l, const float* d_row_u,
                                         float* d_row_viols, const float* d_x, const float* d_c, const float* d_AT_y,
                                         const float* d_l, const float* d_u, const float* d_tau, float* d_col_viols,
                                         void* stream) {
    return guarded([&]() -> int {
        if (m < 0 || n < 0) return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, "negative dimension");
        cudaStream_t s = (cudaStream_t)stream;
        if (m > 0) compat_row_viol_kernel<<<grid_for(m, 256), 256, 0, s>>>(m, d_Ax, d_row_l, d_row_u, d_row_viols);
        if (n > 0)
            compat_col_viol_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, d_x, d_c, d_AT_y, d_l, d_u, d_tau, d_col_viols);
        SIHG_LAUNCH_CHECK();
        return SIH_PDHG_OK;
    });
}
