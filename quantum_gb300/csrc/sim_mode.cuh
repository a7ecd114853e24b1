// One interpreter instantiation of the simulation kernel, compiled in its own
// translation unit per mode so that the modes build in parallel.  The
// including file defines TFQG_SIM_MODE (a SimMode value) and TFQG_SIM_NAME
// (the suffix of the exported launcher names).
//
// The kernel: persistent CTAs pull rows (circuits) or trajectories from a
// work queue.  A row whose state fits shared memory is simulated entirely
// there (resident); larger states live in a per-CTA global slot and are
// streamed through shared memory one tile per pass (the host planner groups
// gates into passes whose targets lie inside the tile).  Epilogues:
// Pauli-sum expectation (util_qsim.h:142-188), state copy with -2 padding
// (tfq_simulate_state_op.cc:196-207), sampling with the reference bit layout
// (tfq_simulate_samples_op.cc:226-243), adjoint sweep
// (tfq_adj_grad_op.cc:199-276), noisy trajectories
// (tfq_noisy_expectation.cc:258-391).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sim_device.cuh"

#define TFQG_CAT2(a, b) a##b
#define TFQG_CAT(a, b) TFQG_CAT2(a, b)

namespace tfqg {

__global__ void __launch_bounds__(kSimThreads, 1)
TFQG_CAT(TFQG_CAT(simulate_, TFQG_SIM_NAME), _kernel)(BatchDevice b, RunArgs a,
                                                      int state_amps, int nstates) {
  simulate_body<TFQG_SIM_MODE, InterpExec>(b, a, state_amps, nstates);
}

const void* TFQG_CAT(sim_kernel_, TFQG_SIM_NAME)() {
  return reinterpret_cast<const void*>(
      &TFQG_CAT(TFQG_CAT(simulate_, TFQG_SIM_NAME), _kernel));
}

cudaError_t TFQG_CAT(sim_launch_, TFQG_SIM_NAME)(const BatchDevice& b, const RunArgs& a,
                                                 int grid, size_t smem, int state_amps,
                                                 int nstates, cudaStream_t s) {
  TFQG_CAT(TFQG_CAT(simulate_, TFQG_SIM_NAME), _kernel)<<<grid, kSimThreads, smem, s>>>(
      b, a, state_amps, nstates);
  return cudaGetLastError();
}

}  // namespace tfqg
