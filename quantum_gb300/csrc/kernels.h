// Launch interface of the sm_103a kernels (kernels.cu), used by the C ABI.
#pragma once
#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#include <stdint.h>
#endif

#include "tfqg_types.h"

namespace tfqg {

enum SimMode { kModeExpect = 0, kModeState, kModeSample, kModeAdjoint, kModeNoisy };

// Device copies of a compiled batch (all pointers are device pointers).
struct BatchDevice {
  const DevProgram* programs = nullptr;
  const DevRow* rows = nullptr;
  const GateTemplate* gates = nullptr;
  const DevPass* passes = nullptr;
  const DevOp* ops = nullptr;
  const DevTerm* terms = nullptr;
  const DevChannel* channels = nullptr;
  const float2* kraus = nullptr;
  const int32_t* grad_cols = nullptr;
  const int32_t* order = nullptr;  // rows, most expensive first
  const DevMeas* meas = nullptr;
  const DevMeasTerm* meas_terms = nullptr;
  int32_t num_rows = 0;
  int32_t num_ops = 0;       // pauli_sums columns
  int32_t num_symbols = 0;
  int32_t max_n = 0;
  int64_t total_gates = 0;   // matrix slots over all rows
  int64_t total_grads = 0;   // derivative slots over all rows
};

struct RunArgs {
  const float* values = nullptr;     // [rows, num_symbols]
  float2* mats = nullptr;            // [total_gates][16]
  float2* dmats = nullptr;           // [total_grads][16]
  float2* work = nullptr;            // per-CTA state slots
  int64_t slot_amps = 0;             // amplitudes per CTA slot
  int* counter = nullptr;            // work-queue counter (zeroed per launch)
  float* out_f = nullptr;            // expectations [rows, ops] / grads [rows, P]
  float2* out_state = nullptr;       // [rows, 2^max_n]
  int8_t* out_samples = nullptr;     // [rows, S, max_n]
  int num_samples = 0;
  const float* dgrads = nullptr;     // [rows, ops]
  const int32_t* reps = nullptr;     // [rows, ops] trajectories per op
  double* acc = nullptr;             // [rows, ops] noisy sums
  const int64_t* traj_prefix = nullptr;  // [rows + 1] trajectory prefix
  int64_t total_traj = 0;
  uint64_t seed = 0;
  int grad_rule = 0;                 // 0: reference finite difference, 1: exact
  int* error_flag = nullptr;         // device word; nonzero = kernel-side error
};

// Threads per CTA of the simulation kernel.
constexpr int kSimThreads = 512;

#ifndef __CUDACC_RTC__
cudaError_t launch_build_matrices(const BatchDevice& b, const RunArgs& a,
                                  bool with_grads, cudaStream_t s);
// Shared memory (bytes) the simulation kernel needs for this batch.
size_t sim_smem_bytes(int mode, int max_resident_n, bool any_streamed,
                      int max_grads);
int sim_state_amps(int max_resident_n, bool any_streamed);
int sim_grid_size(int mode, size_t smem);
cudaError_t launch_simulate(int mode, const BatchDevice& b, const RunArgs& a,
                            int grid, size_t smem, int state_amps,
                            cudaStream_t s);
cudaError_t launch_noisy_finalize(const BatchDevice& b, const RunArgs& a,
                                  cudaStream_t s);

// Per-mode interpreter kernels (sim_<mode>.cu): kernel address and launcher.
#define TFQG_SIM_DECL(name)                                                     \
  const void* sim_kernel_##name();                                              \
  cudaError_t sim_launch_##name(const BatchDevice& b, const RunArgs& a, int grid, \
                                size_t smem, int state_amps, int nstates,       \
                                cudaStream_t s);
TFQG_SIM_DECL(expect)
TFQG_SIM_DECL(state)
TFQG_SIM_DECL(sample)
TFQG_SIM_DECL(adjoint)
TFQG_SIM_DECL(noisy)
#undef TFQG_SIM_DECL
#endif  // __CUDACC_RTC__

}  // namespace tfqg
