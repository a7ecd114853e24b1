// Batch-specialized sub-pass code compiled at run time (jit.cc).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "kernels.h"

struct tfqg_batch;

namespace tfqg {

// Specialized modules: one per SimMode (0..4), plus the wide-row forward pass.
constexpr int kJitWide = 5;
constexpr int kJitModes = 6;

// Records each sub-pass header's signature id (host only; cheap).
void jit_assign_signatures(tfqg_batch* b);
// Generated CUDA source of the batch's executors and kernels.
std::string jit_source(const tfqg_batch* b, int mode);
bool jit_enabled_for(const tfqg_batch* b);
// Specialized kernel for `mode` on device `dev`, or nullptr (interpreter).
cudaKernel_t jit_kernel(tfqg_batch* b, int mode, int dev);
int jit_compile_check(tfqg_batch* b, int mode, std::string* log);
int jit_grid(cudaKernel_t k, size_t smem, int dev, int threads);
int jit_threads(int mode);
cudaError_t jit_launch(cudaKernel_t k, const BatchDevice& bd, const RunArgs& a,
                       int grid, size_t smem, int state_amps, int nstates,
                       cudaStream_t s, int threads);
cudaError_t jit_launch_wide(cudaKernel_t k, const BatchDevice& bd, const RunArgs& a,
                            int row, int pass, int init, float2* psi, int grid,
                            size_t smem, int state_amps, cudaStream_t s);

}  // namespace tfqg
