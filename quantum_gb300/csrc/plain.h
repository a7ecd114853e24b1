// Plain one-launch-per-gate comparison path (plain.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tfqg_types.h"

namespace tfqg {

// A batch whose rows all run the same program and observables.
struct PlainJob {
  int rows = 0, n = 0, num_gates = 0, num_grads = 0, num_terms = 0;
  int n_ops = 0, num_symbols = 0;
  const GateTemplate* gates = nullptr;  // host
  const DevTerm* terms = nullptr;       // host
  const int32_t* grad_cols = nullptr;   // host
  const float2* mats = nullptr;         // device [rows][num_gates][16]
  const float2* dmats = nullptr;        // device [rows][num_grads][16]
  float2* psi = nullptr;                // device [rows][2^n]
  float2* lam = nullptr;                // device [rows][2^n]
  const float* dgrads = nullptr;        // device [rows][n_ops]
  double* acc_exp = nullptr;            // device, zeroed
  double* acc_grad = nullptr;           // device, zeroed
  float* out_exp = nullptr;             // device [rows][n_ops]
  float* out_grad = nullptr;            // device [rows][num_symbols]
};

cudaError_t plain_expect_adjoint(const PlainJob& j, cudaStream_t s,
                                 int64_t* launches);

}  // namespace tfqg

extern "C" {
int64_t tfqg_internal_batch_table_bytes(void* batch);
int tfqg_internal_jit_compile_check(void* batch, int mode, char* err, int64_t err_size);
int64_t tfqg_internal_jit_source(void* batch, int mode, char* buf, int64_t size);
int tfqg_internal_batch_jit(void* batch, int mode, int32_t* nsig, int32_t* active,
                            char* err, int64_t err_size);
int tfqg_internal_batch_subpasses(void* batch, int32_t* fwd_subs,
                                  int32_t* fwd_ops, int32_t* bwd_subs,
                                  int32_t* bwd_ops);
int tfqg_internal_batch_passes(void* batch, int32_t* fwd, int32_t* bwd,
                               int32_t* resident);
// Estimated simulation cost of each row (gates x 2^n amplitude updates; 0
// for empty programs), used to shard a batch across devices.
int tfqg_internal_batch_row_costs(void* batch, double* costs);
int tfqg_internal_set_wide_min_qubits(int n);
int tfqg_internal_set_wide_few_rows(int rows);
int tfqg_internal_set_gate_fusion(int on);
// tcgen05 self-check (tc_mma.cu): D[128x64] = A[128x32] * B[64x32]^T, tf32.
int tfqg_internal_tc_gemm_tf32(const float* A, const float* B, float* D, int* status,
                               void* stream);
int tfqg_internal_program_cache(int on, int64_t* hits, int64_t* misses);
int tfqg_internal_row_sweeps(void* batch, int64_t row, int32_t* fwd, int32_t* meas);
int tfqg_internal_forward_plan_gates(void* batch, int64_t row,
                                     const float* row_values, int32_t* meta,
                                     float* mats, int64_t max, int64_t* count);
uint64_t tfqg_internal_batch_fingerprint(void* batch);
int tfqg_internal_batch_wide_rows(void* batch);
// Expectation + adjoint gradient of a uniform batch by the plain path, all
// buffers on the device.  Used by bench.py as the comparison baseline.
int tfqg_internal_plain_expect_adj(void* batch, const float* symbol_values,
                                   const float* downstream_grads,
                                   float* expectations, float* grads,
                                   void* stream, int64_t* launches);
}
