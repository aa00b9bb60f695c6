// Shared helpers of the sm_103a PDHG engine: error plumbing, device memory
// RAII, warp/block reductions, compensated (two-sum) arithmetic.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "sih_pdhg.h"

namespace sihg {

// ---------------------------------------------------------------- errors
void set_last_error(const std::string& msg);

struct Status {
    int code = SIH_PDHG_OK;
    bool ok() const { return code == SIH_PDHG_OK; }
};

inline int fail(int code, const std::string& msg) {
    set_last_error(msg);
    return code;
}

// Runs an entry point's body so that no C++ exception crosses the C ABI:
// std::bad_alloc becomes SIH_PDHG_ERR_OUT_OF_MEMORY, any other exception
// SIH_PDHG_ERR_INVALID_ARGUMENT with its message.
template <class F>
int guarded(F&& body) {
    try {
        return body();
    } catch (const std::bad_alloc&) {
        return fail(SIH_PDHG_ERR_OUT_OF_MEMORY, "out of host memory");
    } catch (const std::exception& e) {
        return fail(SIH_PDHG_ERR_INVALID_ARGUMENT, std::string("unexpected error: ") + e.what());
    }
}

inline int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    return fail(e == cudaErrorMemoryAllocation ? SIH_PDHG_ERR_OUT_OF_MEMORY : SIH_PDHG_ERR_CUDA, buf);
}

#define SIHG_CUDA(call)                                                   \
    do {                                                                  \
        cudaError_t e_ = (call);                                          \
        if (e_ != cudaSuccess) return ::sihg::cuda_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)

#define SIHG_LAUNCH_CHECK()                                               \
    do {                                                                  \
        cudaError_t e_ = cudaGetLastError();                              \
        if (e_ != cudaSuccess) return ::sihg::cuda_fail(e_, "kernel launch", __FILE__, __LINE__); \
    } while (0)

#define SIHG_TRY(expr)                   \
    do {                                 \
        int rc_ = (expr);                \
        if (rc_ != SIH_PDHG_OK) return rc_; \
    } while (0)

// ---------------------------------------------------------------- device memory
// Owning device allocation (cudaMalloc / cudaFree), movable, never copied.
class DevMem {
  public:
    DevMem() = default;
    DevMem(const DevMem&) = delete;
    DevMem& operator=(const DevMem&) = delete;
    DevMem(DevMem&& o) noexcept : p_(o.p_), bytes_(o.bytes_) { o.p_ = nullptr; o.bytes_ = 0; }
    DevMem& operator=(DevMem&& o) noexcept {
        if (this != &o) { release(); p_ = o.p_; bytes_ = o.bytes_; o.p_ = nullptr; o.bytes_ = 0; }
        return *this;
    }
    ~DevMem() { release(); }
    int alloc(size_t bytes) {
        release();
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMalloc(&p_, bytes);
        if (e != cudaSuccess) { p_ = nullptr; return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__); }
        bytes_ = bytes;
        return SIH_PDHG_OK;
    }
    void release() {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        bytes_ = 0;
    }
    template <class T> T* as() const { return static_cast<T*>(p_); }
    size_t bytes() const { return bytes_; }

  private:
    void* p_ = nullptr;
    size_t bytes_ = 0;
};

// ---------------------------------------------------------------- device helpers
constexpr unsigned FULL_MASK = 0xffffffffu;

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL_MASK, v, o));
    return v;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

__device__ __forceinline__ double warp_maxd(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL_MASK, v, o));
    return v;
}

// Block-wide max of non-negative floats, result valid in thread 0.
// `smem` must hold blockDim.x / 32 floats.
__device__ __forceinline__ float block_max_nonneg(float v, float* smem) {
    v = warp_max(v);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) smem[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? smem[lane] : 0.0f;
        v = warp_max(v);
    }
    __syncthreads();
    return v;
}

// Knuth's two-sum: s + e == a + b exactly (round-to-nearest).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Two-product via fused multiply-add: p + e == a * b exactly.
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

// Compensated FP32 accumulator (Neumaier summation built on two-sum): the
// running value is s + c with an error of about eps^2 relative to the sum of
// magnitudes.  Per-element reductions use it so that FP64 (a slow pipe on this
// part) is only touched once per thread at the block reduction.
struct Acc {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        float t, e;
        two_sum(s, v, t, e);
        s = t;
        c = __fadd_rn(c, e);
    }
    // adds a * b exactly (two-product)
    __device__ __forceinline__ void add_prod(float a, float b) {
        float p, e;
        two_prod(a, b, p, e);
        add(p);
        c = __fadd_rn(c, e);
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
    __device__ __forceinline__ void reset() { s = c = 0.f; }
};

// Float-float number hi + lo (about 48 significant bits): the running averages.
__device__ __forceinline__ float2 ff_axpy(float2 acc, float w, float x) {
    // acc + w * (x - acc), evaluated in float-float arithmetic
    float d_hi, d_lo;
    two_sum(x, -acc.x, d_hi, d_lo);
    d_lo = __fsub_rn(d_lo, acc.y);
    const float d = __fadd_rn(d_hi, d_lo);
    float p, pe;
    two_prod(w, d, p, pe);
    float s, se;
    two_sum(acc.x, p, s, se);
    const float lo = __fadd_rn(__fadd_rn(acc.y, se), pe);
    float hi2, lo2;
    two_sum(s, lo, hi2, lo2);
    return make_float2(hi2, lo2);
}

}  // namespace sihg
