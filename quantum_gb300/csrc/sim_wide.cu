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
