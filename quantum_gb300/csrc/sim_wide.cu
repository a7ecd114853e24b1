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

// Lockstep rows: one forward pass of every row of a group (items[i].pass of
// row items[i].row), tile by tile over the whole grid; the state of a row is
// its output row (tfq_simulate_state) or arena + items[i].off.  `init`
// starts each row from |0...0> instead of loading its state.
__global__ void __launch_bounds__(kWideThreads, 2)
simulate_lock_pass_kernel(BatchDevice b, RunArgs a, const LockItem* items, int nitems,
                          int64_t ntiles, float2* arena, int init, int to_out_state,
                          int state_amps) {
  const Smem sm = carve_smem<kModeState>(state_amps, 1);
  int kc = 0;  // sub-pass counter (staging buffer parity)
  for (int64_t T = blockIdx.x; T < ntiles; T += gridDim.x) {
    int lo = 0, hi = nitems - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (items[mid].prefix <= T) lo = mid;
      else hi = mid - 1;
    }
    const LockItem it = items[lo];
    RowCtx rc;
    rc.row = it.row;
    rc.traj = 0;
    rc.r = b.rows[it.row];
    rc.p = b.programs[rc.r.program];
    const int n = rc.p.n;
    float2* psi = to_out_state ? a.out_state + (int64_t(it.row) << b.max_n) : arena + it.off;
    const DevPass ps = b.passes[it.pass];
    build_hi_table(sm.hi, ps.tile_mask);
    __syncthreads();
    const uint32_t all = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
    const uint32_t base = deposit(uint32_t(T - it.prefix), all & ~ps.tile_mask);
    if (init) tile_zero(sm.psi, base == 0);
    else tile_load_async(sm.psi, psi, sm.hi, base);
    tile_load_wait();
    __syncthreads();
    run_ops<kModeState, InterpExec>(b, a, sm, rc, ps.op_begin, ps.op_end, sm.psi, sm.lam,
                                    kTile, base, kc);
    tile_store(psi, sm.psi, sm.hi, base);
    __syncthreads();
  }
}

const void* sim_kernel_lock() {
  return reinterpret_cast<const void*>(&simulate_lock_pass_kernel);
}

cudaError_t sim_launch_lock(const BatchDevice& b, const RunArgs& a, const LockItem* items,
                            int nitems, int64_t ntiles, float2* arena, int init,
                            int to_out_state, int grid, size_t smem, int state_amps,
                            cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  simulate_lock_pass_kernel<<<grid, kWideThreads, smem, s>>>(
      b, a, items, nitems, ntiles, arena, init, to_out_state, state_amps);
  return cudaGetLastError();
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
