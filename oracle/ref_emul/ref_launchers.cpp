/*
 * Runs the reference's PDHG kernels (core/src/gpu/cuda_pdhg.cu:11-151) on the
 * CPU.  The kernel definitions are taken verbatim from the reference file by
 * oracle/ref_build.sh into oracle/_ref/ (git-ignored) and included here; each
 * launcher below has the signature that gpu_solver.cpp:18-40 declares and
 * calls its kernel once per (block, thread) of the grid the reference
 * launchers use (cuda_pdhg.cu:155-203: 256 threads per block).
 * TEST INFRASTRUCTURE ONLY.
 */
#define SIH_CUDA_ENABLED 1
#include "cuda_runtime.h"

dim3 blockDim, blockIdx, threadIdx;

#include "ref_kernels.inc"

template <class F>
static void emulate_grid(int n_threads_total, F&& body) {
    const unsigned bs = 256;
    const unsigned gs = (unsigned)((n_threads_total + (int)bs - 1) / (int)bs);
    blockDim = dim3{bs, 1, 1};
    for (unsigned b = 0; b < gs; ++b)
        for (unsigned t = 0; t < bs; ++t) {
            blockIdx = dim3{b, 0, 0};
            threadIdx = dim3{t, 0, 0};
            body();
        }
}

void launch_csr_spmv(int m, const int* d_row_ptr, const int* d_col_ind, const float* d_values, const float* d_x,
                     float* d_y, cudaStream_t) {
    emulate_grid(m, [&] { csr_spmv_kernel(m, d_row_ptr, d_col_ind, d_values, d_x, d_y); });
}
void launch_csc_spmv(int n, const int* d_col_ptr, const int* d_row_ind, const float* d_values, const float* d_y,
                     float* d_z, cudaStream_t) {
    emulate_grid(n, [&] { csc_spmv_kernel(n, d_col_ptr, d_row_ind, d_values, d_y, d_z); });
}
void launch_primal_update(int n, const float* d_tau, const float* d_c, const float* d_AT_y, const float* d_l,
                          const float* d_u, float* d_x, float* d_x_bar, cudaStream_t) {
    emulate_grid(n, [&] { primal_update_kernel(n, d_tau, d_c, d_AT_y, d_l, d_u, d_x, d_x_bar); });
}
void launch_dual_update(int m, const float* d_sigma, const float* d_A_xbar, const float* d_row_l,
                        const float* d_row_u, float* d_y, cudaStream_t) {
    emulate_grid(m, [&] { dual_update_kernel(m, d_sigma, d_A_xbar, d_row_l, d_row_u, d_y); });
}
void launch_restart(int n, const float* d_x, float* d_x_bar, cudaStream_t) {
    emulate_grid(n, [&] { restart_kernel(n, d_x, d_x_bar); });
}
void launch_residuals(int m, int n, const float* d_Ax, const float* d_row_l, const float* d_row_u,
                      float* d_row_viols, const float* d_x, const float* d_c, const float* d_AT_y, const float* d_l,
                      const float* d_u, const float* d_tau, float* d_col_viols, cudaStream_t) {
    emulate_grid(m, [&] { row_residuals_kernel(m, d_Ax, d_row_l, d_row_u, d_row_viols); });
    emulate_grid(n, [&] { col_residuals_kernel(n, d_x, d_c, d_AT_y, d_l, d_u, d_tau, d_col_viols); });
}

}  // namespace gpu
}  // namespace sih
