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
  const int32_t* order = nullptr;  // rows the persistent kernel takes, most
                                   // expensive first (num_queue of them)
  const DevMeas* meas = nullptr;
  const DevMeasTerm* meas_terms = nullptr;
  int32_t num_rows = 0;
  int32_t num_queue = 0;     // entries of `order` the persistent kernel runs
  int32_t num_ops = 0;       // pauli_sums columns
  int32_t num_symbols = 0;
  int32_t max_n = 0;
  int64_t total_gates = 0;   // matrix slots over all rows
  int64_t total_grads = 0;   // derivative slots over all rows
  int32_t any_fused = 0;     // some program holds GK_FUSED gates
  int32_t pad_ = 0;
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
  // adjoint: lambda seeded from a buffer ([rows, lambda_stride] amplitudes,
  // times i^lambda_rot) instead of from the observables, and the scale of
  // the gradient output (2 for the expectation gradient)
  const float2* lambda_init = nullptr;
  int64_t lambda_stride = 0;
  int lambda_rot = 0;
  float grad_scale = 2.f;
  int sample_terms = 0;              // noisy: each term measured once per trajectory
  double* term_vals = nullptr;       // optional [rows, term_stride]: <psi|P_t|psi>
  int64_t term_stride = 0;           // per term of the row (no coefficient)
};

// Threads per CTA of the simulation kernel.
constexpr int kSimThreads = 512;
// Threads per CTA of the wide-row kernels (two CTAs per SM, so that one
// CTA's tile loads and stores overlap the other's arithmetic).
constexpr int kWideThreads = 256;
// Rows of at least this many qubits run as wide rows in the forward modes:
// the whole grid works on one state, one launch per pass.
constexpr int kWideMinQubits = 22;
// A batch that streams R < kWideFewRows rows runs a row of n >=
// kWideFewQubits qubits as a wide row too when R <= 2^(n-14) (half its
// tiles per pass).
constexpr int kWideFewRows = 64;
constexpr int kWideFewQubits = 17;

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
// tfq_inner_product over the rows of a TFQG_KIND_INNER batch: states holds
// every row's final state (row stride `stride` amplitudes); out[i, j] =
// <psi_i | phi_ij> in complex64 from fp64 sums (`acc`: 2 doubles per pair,
// zeroed by the caller); 1 for an empty reference program.
cudaError_t launch_inner_products(const BatchDevice& b, const float2* states,
                                  int64_t stride, int main_rows, int others,
                                  double* acc, float2* out, cudaStream_t s);

// chi_i = sum_j g_ij phi_ij for the reference rows of a TFQG_KIND_INNER batch
// (AccumulateFusedCircuits, tfq_inner_product_grad.cc:254-258), written over
// the reference rows' states (rows 0..main_rows-1 of `states`).
cudaError_t launch_paired_sum(const BatchDevice& b, float2* states, int64_t stride,
                              int main_rows, int others, const float* grads,
                              cudaStream_t s);
// out[k] = (re[k], -im[k]) as complex64: <dU psi | chi> from the adjoint's
// Re<lambda|dU psi> runs with lambda = chi and lambda = i chi.
cudaError_t launch_conj_combine(const float* re, const float* im, float2* out, int64_t n,
                                cudaStream_t s);

// Sampled expectation from the term values a.term_vals: per (row, op), each
// term's N = num_samples[row, op] measurement parities drawn as Bernoulli
// trials; writes a.out_f.
cudaError_t launch_sampled_expectation(const BatchDevice& b, const RunArgs& a,
                                       const int32_t* num_samples, cudaStream_t s);

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

// Wide rows (kernels.cu, sim_wide.cu).  `psi` is the row's 2^n state in
// global memory; grids are multiples of the SM count.
const void* sim_kernel_wide();
cudaError_t sim_launch_wide(const BatchDevice& b, const RunArgs& a, int row, int pass,
                            int init, float2* psi, int grid, size_t smem,
                            int state_amps, cudaStream_t s);
// Adjoint of a wide row: lambda accumulation per measurement pass, backward
// passes adding gradient-slot sums into gacc (doubles), then the finalize
// into out_f.  psi and lam are the row's two 2^n states.
const void* sim_kernel_wide_lambda();
const void* sim_kernel_wide_backward();
cudaError_t sim_launch_wide_lambda(const BatchDevice& b, const RunArgs& a, int row, int mp,
                                   int first, const float2* psi, float2* lam, int grid,
                                   size_t smem, int state_amps, cudaStream_t s);
cudaError_t sim_launch_wide_backward(const BatchDevice& b, const RunArgs& a, int row,
                                     int pass, float2* psi, float2* lam, double* gacc,
                                     int grid, size_t smem, int state_amps, cudaStream_t s);
cudaError_t launch_wide_grad_finalize(const BatchDevice& b, const RunArgs& a, int row,
                                      const double* gacc, cudaStream_t s);
const void* wide_measure_kernel_ptr();
cudaError_t launch_wide_measure(const BatchDevice& b, const RunArgs& a, int row, int mp,
                                const float2* psi, double* wacc, int term0, int grid,
                                size_t smem, int state_amps, cudaStream_t s);
// out_f[row, :] from the term sums; `scratch` holds num_ops doubles.
cudaError_t launch_wide_expect_finalize(const BatchDevice& b, const RunArgs& a, int row,
                                        const double* wacc, int term0, double* scratch,
                                        cudaStream_t s);
// csum[c] = sum of |psi|^2 over amplitudes [c * 2^13, (c + 1) * 2^13).
cudaError_t launch_wide_chunk_sums(const float2* psi, int n, double* csum, int grid,
                                   cudaStream_t s);
// Draws a.num_samples samples of row `row` from psi using the chunk sums
// (scanned in place) and writes them in the reference bit layout.
cudaError_t launch_wide_sample(const BatchDevice& b, const RunArgs& a, int row,
                               const float2* psi, int n, double* csum, cudaStream_t s);
// Lockstep rows (forward modes): streamed rows of lock_min..21 qubits in a
// batch with many of them run side by side over the whole grid instead of
// one CTA each: launch k runs forward pass k of every row of a group, tile
// by tile (the launch boundary orders the passes), then the measurement
// passes, the expectation finalize or the sampling, all over the group's
// rows at once.  An item is one row of a launch: its pass (forward or
// measurement), the global index of its first tile or chunk (prefix,
// ascending over the items), its state offset in the arena, its qubits and
// the first of its row's term accumulators in the group (acc: rows that
// share a program and observables share their measurement passes, so the
// sums are kept per row, not per measurement term).
struct LockItem {
  int32_t row;
  uint32_t pass;
  int64_t prefix;
  int64_t off;
  int32_t n;
  int32_t acc;
};
static_assert(sizeof(LockItem) == 32, "LockItem layout");
// Lockstep sampling sums |psi|^2 over chunks of 2^kLockChunkBits amplitudes
// (a row item's prefix counts these chunks).
constexpr int kLockChunkBits = 8;
const void* sim_kernel_lock();
cudaError_t sim_launch_lock(const BatchDevice& b, const RunArgs& a, const LockItem* items,
                            int nitems, int64_t ntiles, float2* arena, int init,
                            int to_out_state, int grid, size_t smem, int state_amps,
                            cudaStream_t s);
const void* lock_measure_kernel_ptr();
cudaError_t launch_lock_measure(const BatchDevice& b, const RunArgs& a, const LockItem* items,
                                int nitems, int64_t ntiles, const float2* arena,
                                double* wacc, int grid, size_t smem, int state_amps,
                                cudaStream_t s);
// out_f of the rows; `scratch` holds nrows * num_ops doubles.
cudaError_t launch_lock_expect_finalize(const BatchDevice& b, const RunArgs& a,
                                        const LockItem* rows, int nrows, const double* wacc,
                                        double* scratch, cudaStream_t s);
cudaError_t launch_lock_chunk_sums(const LockItem* rows, int nrows, int64_t nchunks,
                                   const float2* arena, double* csum, int grid,
                                   cudaStream_t s);
cudaError_t launch_lock_sample(const BatchDevice& b, const RunArgs& a, const LockItem* rows,
                               int nrows, const float2* arena, double* csum,
                               cudaStream_t s);
cudaError_t launch_lock_pad(const BatchDevice& b, const RunArgs& a, const LockItem* rows,
                            int nrows, cudaStream_t s);
// Tensor-core forward path (tc_gates.cu).  launch_tc_fuse writes the
// 32 x 32 complex64 matrix of each block (row-major, 1024 entries per block)
// from the row's bound gate matrices `mats`; launch_tc_apply5 applies one
// block's matrix U to the 2^n state psi (n in [12, 31]) over `grid` CTAs and
// sets *status to 1 if an MMA completion wait timed out.
const void* tc_apply5_kernel_ptr();
size_t tc_apply5_smem_bytes();
cudaError_t launch_tc_fuse(const BatchDevice& b, const float2* mats, int row,
                           const TcBlock* blocks, const int32_t* members, int nblocks,
                           float2* U, cudaStream_t s);
cudaError_t launch_tc_apply5(float2* psi, int n, const float2* U, const TcBlock& blk,
                             int* status, int grid, cudaStream_t s);
// Chunk geometry of the block kernel's transposed variant (blocks with a
// target among bits 0-4): the 12 index bits of a chunk in ascending order
// (cb, 5 bits each), the chunk positions of the 7 row bits and the 5
// targets (rpos, tpos, 4 bits each) and the staging-buffer swizzle term of
// chunk positions 4..11 (c, 4 bits each).  Returns false for blocks that
// take the direct variant.
struct TcTrans {
  uint64_t cb;
  uint32_t rpos;
  uint32_t tpos;
  uint32_t c;
};
bool tc_transposed_geometry(const TcBlock& blk, int n, TcTrans* out);
// Two blocks in one sweep over the state (tc_sweep_kernel): tiles of 13
// index bits -- bits 0-2, both blocks' targets and the lowest free bits --
// staged through shared memory by bulk copies (cp.async.bulk, the TMA
// engine) and written back the same way, with both blocks applied to each
// tile on the tensor cores (A operands in tensor memory).  The geometry:
// the physical bit of every tile position (cb, 5 bits each, positions 0-11;
// cb12 position 12), the tile bits as a mask, per block its target and row
// positions (4 bits each), the staging swizzle (tile positions whose parity
// flips 8-byte slot bit 3) and the length r0 of the tile's lowest run of
// consecutive bits.  False when the blocks cannot share a sweep (a target
// below bit 4, or more than 13 tile bits).
struct TcSweep {
  uint64_t cb;
  uint32_t cb12;
  uint32_t smask;
  uint32_t tpos[2];
  uint32_t rpos[2];
  uint32_t hmask;
  uint32_t r0;
};
bool tc_sweep_geometry(const TcBlock& b0, const TcBlock& b1, int n, TcSweep* out);
size_t tc_sweep_smem_bytes();
const void* tc_sweep_kernel_ptr();
// Applies U0 (block b0) then U1 (block b1) to the 2^n state in one sweep;
// `grid` CTAs (one per SM); *status set to 1 on a timed-out wait.
cudaError_t launch_tc_sweep2(float2* psi, int n, const float2* U0, const float2* U1,
                             const TcBlock& b0, const TcBlock& b1, int* status, int grid,
                             cudaStream_t s);
// Lockstep rows on the tensor cores: block k of every row of a lockstep
// group in one launch.  A unit is a run of consecutive chunks (128 groups of
// 32 amplitudes each) of one row's state under one block: the state (arena
// offset `off`, or batch row `row` of the output states), the block's B
// operands (index `mat` among its group's blocks, whose B operands are
// built for each group in turn), its packed targets and, for the
// transposed variant, its chunk geometry.  Units of one launch all take the
// same variant.
// In the persistent form (one launch per group, see
// launch_tc_lock_persistent) a unit also carries the transposed-variant flag
// (tpack bit 31), its row's slot among the batch's tensor-core rows and the
// number of that row's units that must be done before it starts (those of
// the row's earlier blocks).
struct TcUnit {
  int64_t off;
  int64_t chunk0;
  int32_t nchunks;
  int32_t row;
  uint32_t tpack;
  uint32_t mat;
  TcTrans tr;
  int32_t slot;
  int32_t need;
};
static_assert(sizeof(TcUnit) == 64, "TcUnit layout");
constexpr uint32_t kTcUnitTrans = 1u << 31;
// Chunks per unit: at most kTcUnitChunks (one bulk copy of the block's B
// operands per unit), fewer where a launch would have fewer than
// kTcUnitTarget units.  (On GB300, 128 random 17-qubit rows in one
// persistent launch: 3.35 ms per call with these values, 3.57 ms with a
// target of 512 units, 5.05 ms with 2048.)
constexpr int kTcUnitChunks = 16;
constexpr int64_t kTcUnitTarget = 256;
// Targets of `blk` packed 5 bits each and the variant (1 transposed, 0
// direct, with its geometry in *tr), or -1 when the block does not fit a
// 2^n state.
int tc_unit_geometry(const TcBlock& blk, int n, uint32_t* tpack, TcTrans* tr);
// Floats of one block's B operands (R in real form, tf32 hi then lo, in
// the block kernel's shared-memory layout).
size_t tc_b_floats();
// B operands of blocks whose rows differ (block i belongs to batch row
// block_rows[i]), from the member gates' bound matrices in complex64:
// B + i * tc_b_floats().
cudaError_t launch_tc_fuse_b(const BatchDevice& b, const float2* mats,
                             const int32_t* block_rows, const TcBlock* blocks,
                             const int32_t* members, int nblocks, float* B, cudaStream_t s);
// Applies each unit's block (B operands B + mat * tc_b_floats(), 16-byte
// aligned) to its chunks; the state of a unit is state + off, or
// state + (row << row_shift) when row_shift >= 0.  *status set to 1 on a
// timed-out wait.
cudaError_t launch_tc_apply5_units(float2* state, int row_shift, const float* B,
                                   const TcUnit* units, int nunits, bool trans, int* status,
                                   int grid, cudaStream_t s);
// All units of a lockstep group in one launch: CTAs take units in queue
// order from *queue (zeroed before the launch); a unit waits (bounded) until
// done[slot] >= need, runs, then counts itself in done[slot] (zeroed before
// the launch).  A timed-out wait sets *status and every CTA stops taking
// units.
cudaError_t launch_tc_lock_persistent(float2* state, int row_shift, const float* B,
                                      const TcUnit* units, int nunits, int* queue, int* done,
                                      int* status, int grid, cudaStream_t s);
// |0...0> in every row of `rows` (chunks of 2^kLockChunkBits amplitudes
// counted by the items' prefixes); states at arena + off, or at
// state + (row << row_shift) when row_shift >= 0.
cudaError_t launch_lock_zero(float2* state, int row_shift, const LockItem* rows, int nrows,
                             int64_t nchunks, int grid, cudaStream_t s);
// After a captured call whose tensor-core launches set *status: the rows'
// results are replaced by markers (expectations and amplitudes NaN, every
// sample -1), since a replay has no host check.  Does nothing while
// *status is 0.
cudaError_t launch_lock_tc_poison(const BatchDevice& b, const RunArgs& a, int mode,
                                  const LockItem* rows, int nrows, const int* status,
                                  cudaStream_t s);
// p[i] = (i == 0 ? first : rest) for i in [0, count).
cudaError_t launch_fill(float2* p, int64_t count, float2 first, float2 rest, int grid,
                        cudaStream_t s);
#endif  // __CUDACC_RTC__

}  // namespace tfqg
