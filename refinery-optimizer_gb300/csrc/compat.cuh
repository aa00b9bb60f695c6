// Kernels of the reference-compatible launchers (compat.cu), declared for
// reuse by other translation units.
#pragma once

namespace sihg {

__global__ void split_spmv_kernel(int nseg, const int* __restrict__ ptr, const int* __restrict__ idx,
                                  const float* __restrict__ val, const float* __restrict__ vec,
                                  float* __restrict__ out, int L);
__global__ void compat_row_viol_kernel(int m, const float* __restrict__ ax, const float* __restrict__ rl,
                                       const float* __restrict__ ru, float* __restrict__ out);
__global__ void compat_col_viol_kernel(int n, const float* __restrict__ x, const float* __restrict__ c,
                                       const float* __restrict__ aty, const float* __restrict__ l,
                                       const float* __restrict__ u, const float* __restrict__ tau,
                                       float* __restrict__ out);

}  // namespace sihg
