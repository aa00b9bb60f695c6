/*
 * Host-only stand-in for the few CUDA runtime calls that the reference GPU
 * driver (core/src/gpu/gpu_solver.cpp) and kernels (core/src/gpu/cuda_pdhg.cu)
 * use, so that the reference's own PDHG code can run on a CPU to produce
 * golden vectors.  TEST INFRASTRUCTURE ONLY: it is used by oracle/ref_build.sh
 * and by nothing that ships.
 *
 * "Device" memory is host memory; kernels become plain functions that
 * ref_launchers.cpp calls once per (block, thread) of the launch grid.
 *
 * With SIH_EMUL_INTENDED_INDEX_COPY defined, a copy whose source is an int64
 * array converts each element to int32 instead of copying raw bytes.  This is
 * the copy the reference meant at gpu_solver.cpp:202-203 (its int64 CSC arrays
 * go into int32 device buffers, sized as int32).  Without the macro the bytes
 * are copied as the shipped code does, which reproduces its corrupted A^T y.
 */
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>

typedef int cudaError_t;
enum { cudaSuccess = 0 };
typedef struct sih_emul_stream* cudaStream_t;
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3
};

struct dim3 {
    unsigned x, y, z;
};
extern dim3 blockDim, blockIdx, threadIdx;

#define __global__

inline cudaError_t cudaGetDeviceCount(int* count) {
    *count = 1;
    return cudaSuccess;
}
inline cudaError_t cudaMemGetInfo(size_t* free_b, size_t* total_b) {
    *free_b = (size_t)1 << 33;
    *total_b = (size_t)1 << 33;
    return cudaSuccess;
}
template <class T>
inline cudaError_t cudaMalloc(T** ptr, size_t bytes) {
    *ptr = static_cast<T*>(std::malloc(bytes ? bytes : 1));
    return cudaSuccess;
}
inline cudaError_t cudaFree(void* ptr) {
    std::free(ptr);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void* dst, const void* src, size_t bytes, cudaMemcpyKind) {
    std::memcpy(dst, src, bytes);
    return cudaSuccess;
}
#ifdef SIH_EMUL_INTENDED_INDEX_COPY
inline cudaError_t cudaMemcpy(void* dst, const int64_t* src, size_t bytes, cudaMemcpyKind) {
    int* out = static_cast<int*>(dst);
    for (size_t k = 0; k < bytes / sizeof(int); ++k) out[k] = static_cast<int>(src[k]);
    return cudaSuccess;
}
#endif
