// Interpreter kernel of one forward pass of a wide row (a state too large for
// one CTA): every CTA takes a strided share of the pass's tiles.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sim_device.cuh"

namespace tfqg {

__global__ void __launch_bounds__(kWideThreads, 2)
simulate_wide_pass_kernel(BatchDevice b, RunArgs a, int row, int pass, int init,
                          float2* psi, int state_amps) {
  wide_pass_body<InterpExec>(b, a, row, pass, init, psi, state_amps);
}

// Wide rows in the adjoint (interpreter): lambda accumulation and backward
// passes, one launch per pass, then the gradient finalize.
__global__ void __launch_bounds__(kSimThreads, 1)
simulate_wide_lambda_kernel(BatchDevice b, RunArgs a, int row, int mp, int first,
                            const float2* psi, float2* lam, int state_amps) {
  wide_lambda_body(b, a, row, mp, first, psi, lam, state_amps);
}

__global__ void __launch_bounds__(kSimThreads, 1)
simulate_wide_backward_kernel(BatchDevice b, RunArgs a, int row, int pass, float2* psi,
                              float2* lam, double* gacc, int state_amps) {
  wide_backward_body<InterpExec>(b, a, row, pass, psi, lam, gacc, state_amps);
}

// out[row, symbol] += grad_scale * gacc[slot] for every derivative slot, in
// slot order (one thread: deterministic, as the persistent kernel's sum).
__global__ void wide_grad_finalize_kernel(BatchDevice b, RunArgs a, int row,
                                          const double* gacc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const DevProgram p = b.programs[b.rows[row].program];
  float* out = a.out_f + int64_t(row) * b.num_symbols;
  for (int k = 0; k < p.num_grads; ++k)
    out[b.grad_cols[p.grad_col_begin + k]] += float(double(a.grad_scale) * gacc[k]);
}

const void* sim_kernel_wide_lambda() {
  return reinterpret_cast<const void*>(&simulate_wide_lambda_kernel);
}
const void* sim_kernel_wide_backward() {
  return reinterpret_cast<const void*>(&simulate_wide_backward_kernel);
}

cudaError_t sim_launch_wide_lambda(const BatchDevice& b, const RunArgs& a, int row, int mp,
                                   int first, const float2* psi, float2* lam, int grid,
                                   size_t smem, int state_amps, cudaStream_t s) {
  simulate_wide_lambda_kernel<<<grid, kSimThreads, smem, s>>>(b, a, row, mp, first, psi,
                                                               lam, state_amps);
  return cudaGetLastError();
}

cudaError_t sim_launch_wide_backward(const BatchDevice& b, const RunArgs& a, int row,
                                     int pass, float2* psi, float2* lam, double* gacc,
                                     int grid, size_t smem, int state_amps, cudaStream_t s) {
  simulate_wide_backward_kernel<<<grid, kSimThreads, smem, s>>>(b, a, row, pass, psi, lam,
                                                                 gacc, state_amps);
  return cudaGetLastError();
}

cudaError_t launch_wide_grad_finalize(const BatchDevice& b, const RunArgs& a, int row,
                                      const double* gacc, cudaStream_t s) {
  wide_grad_finalize_kernel<<<1, 32, 0, s>>>(b, a, row, gacc);
  return cudaGetLastError();
}

const void* sim_kernel_wide() {
  return reinterpret_cast<const void*>(&simulate_wide_pass_kernel);
}

cudaError_t sim_launch_wide(const BatchDevice& b, const RunArgs& a, int row, int pass,
                            int init, float2* psi, int grid, size_t smem,
                            int state_amps, cudaStream_t s) {
  simulate_wide_pass_kernel<<<grid, kWideThreads, smem, s>>>(b, a, row, pass, init, psi,
                                                              state_amps);
  return cudaGetLastError();
}

}  // namespace tfqg
