/*
 * tfq_gb300: C ABI of the GB300 (sm_103a) implementation of TensorFlow
 * Quantum's state-vector ops.
 *
 * Each entry point replaces the Compute() of one reference TF op kernel;
 * inputs keep the reference's meaning:
 *   programs       serialized tfq.proto.Program, one per batch row
 *   symbol_names   symbol names, one per column of symbol_values
 *   symbol_values  float32 [batch, num_symbols], row-major
 *   pauli_sums     serialized tfq.proto.PauliSum, [batch, num_ops] row-major
 * Strings are passed as arrays of (pointer, length); nothing is retained
 * after a call returns except inside a tfqg_batch handle.
 *
 * Errors: every function returns a tensorflow::error::Code value
 * (0 = OK, 3 = INVALID_ARGUMENT, 8 = RESOURCE_EXHAUSTED, 12 = UNIMPLEMENTED,
 * 13 = INTERNAL).  tfqg_last_error() returns the message of the last failed
 * call on the calling thread; the texts of INVALID_ARGUMENT errors are the
 * reference's.
 *
 * Buffers: functions taking `device_buffers` read inputs and write outputs
 * through device pointers when it is nonzero (asynchronously on `stream`),
 * else through host pointers (the call copies and synchronizes).  `stream`
 * is a cudaStream_t or NULL for the legacy default stream.
 */
#ifndef TFQ_GB300_H_
#define TFQ_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TFQG_OK 0
#define TFQG_INVALID_ARGUMENT 3
#define TFQG_RESOURCE_EXHAUSTED 8
#define TFQG_UNIMPLEMENTED 12
#define TFQG_INTERNAL 13

/* Batch kinds (what the batch will be run for). */
#define TFQG_KIND_FORWARD 0 /* expectation / state / samples */
#define TFQG_KIND_ADJOINT 1 /* adjoint gradient (and forward) */
#define TFQG_KIND_NOISY 2   /* noisy trajectories (channels allowed) */
#define TFQG_KIND_INNER 3   /* tfq_inner_product (tfqg_batch_create_inner_product) */

/* Derivative rule of the adjoint gradient. */
#define TFQG_GRAD_REFERENCE_FD 0 /* (G(x+5e-3)-G(x-5e-3))/1e-2, adj_util.cc:32 */
#define TFQG_GRAD_EXACT 1        /* exact dG/dx */

const char* tfqg_last_error(void);
const char* tfqg_version(void);

/* ---------------------------------------------------------------------
 * Compiled batch: parse + qubit/symbol resolution + pass planning once,
 * run many times with new symbol values.  Creation touches no GPU.
 * ------------------------------------------------------------------- */
typedef struct tfqg_batch tfqg_batch;

/* Parses programs and pauli_sums (pauli_sums may be NULL with num_ops = 0)
 * and resolves symbols.  Mirrors the parse/validation part of
 *   TfqSimulateExpectationOp::Compute  tfq_simulate_expectation_op.cc:50-114
 *   TfqAdjointGradientOp::Compute      tfq_adj_grad_op.cc:51-129
 *   TfqNoisyExpectationOp::Compute     noise/tfq_noisy_expectation.cc:62-135
 * (GetProgramsAndNumQubits parse_context.cc:268-320, GetSymbolMaps :405-461,
 * QsimCircuitFromProgram circuit_parser_qsim.cc:828-861). */
int tfqg_batch_create(const char* const* programs, const int64_t* program_lens,
                      int64_t batch, const char* const* symbol_names,
                      const int64_t* symbol_name_lens, int64_t num_symbols,
                      const char* const* pauli_sums,
                      const int64_t* pauli_sum_lens, int64_t num_ops, int kind,
                      tfqg_batch** out);

/* Largest qubit count in the batch (output width of state / samples). */
int tfqg_batch_max_num_qubits(const tfqg_batch* b, int32_t* out);
/* Synchronizes the batch's device and frees the batch.  Its device buffers
 * return to a process-wide pool that later batches draw from (capped by
 * TFQG_POOL_MAX_BYTES, default 4 GiB; 0 disables the pool). */
void tfqg_batch_destroy(tfqg_batch* b);

/* Frees every pooled device block and empties the process-wide cache of
 * compiled programs (keyed by program bytes, symbol names, batch kind).  No
 * reference counterpart: the reference re-parses and re-allocates per op
 * call, which is what these caches save. */
void tfqg_release_cached_memory(void);

/* Expectations [batch, num_ops]; -2 for empty programs.
 * Replaces TfqSimulateExpectationOp::ComputeSmall/Large
 * (tfq_simulate_expectation_op.cc:130-250). */
int tfqg_batch_expectation(tfqg_batch* b, const float* symbol_values,
                           float* expectations, int device_buffers,
                           void* stream);

/* States complex64 [batch, 2^max_num_qubits] (interleaved float re, im),
 * padded with -2.  Replaces TfqSimulateStateOp (tfq_simulate_state_op.cc:
 * 120-215). */
int tfqg_batch_state(tfqg_batch* b, const float* symbol_values, void* states,
                     int device_buffers, void* stream);

/* Samples int8 [batch, num_samples, max_num_qubits]; padding -2 in the
 * leading columns.  Replaces TfqSimulateSamplesOp
 * (tfq_simulate_samples_op.cc:132-251).  num_samples must be >= 0. */
int tfqg_batch_samples(tfqg_batch* b, const float* symbol_values,
                       int32_t num_samples, uint64_t seed, int8_t* samples,
                       int device_buffers, void* stream);

/* Adjoint gradient [batch, num_symbols] of sum_j downstream_grads[i, j] *
 * <pauli_sums[i, j]>.  Replaces TfqAdjointGradientOp::ComputeSmall/Large
 * (tfq_adj_grad_op.cc:173-390).  The batch must be TFQG_KIND_ADJOINT. */
int tfqg_batch_adj_grad(tfqg_batch* b, const float* symbol_values,
                        const float* downstream_grads, int grad_rule,
                        float* grads, int device_buffers, void* stream);

/* Monte-Carlo trajectory expectations [batch, num_ops]; num_samples int32
 * [batch, num_ops] trajectories per entry (each >= 1).  Replaces
 * TfqNoisyExpectationOp::ComputeSmall/Large (noise/tfq_noisy_expectation.cc:
 * 161-391).  The batch must be TFQG_KIND_NOISY. */
int tfqg_batch_noisy_expectation(tfqg_batch* b, const float* symbol_values,
                                 const int32_t* num_samples, uint64_t seed,
                                 float* expectations, int device_buffers,
                                 void* stream);

/* Sampled expectations [batch, num_ops]; num_samples int32 [batch, num_ops]
 * measurement samples per Pauli term of each entry (each >= 1).  Replaces
 * TfqSimulateSampledExpectationOp::Compute (tfq_simulate_sampled_expectation_
 * op.cc:50-312; util_qsim.h:199-270): per term, the parities of num_samples
 * measurements in the term's basis, averaged and weighted by the real
 * coefficient; identity terms add their coefficient; empty programs give -2.
 * The parities are drawn from the exact <P> (same distribution as sampling
 * the rotated state).  FORWARD or ADJOINT batches with pauli sums. */
int tfqg_batch_sampled_expectation(tfqg_batch* b, const float* symbol_values,
                                   const int32_t* num_samples, uint64_t seed,
                                   float* expectations, int device_buffers,
                                   void* stream);

/* tfq_inner_product batches (TFQG_KIND_INNER).  other_programs holds
 * batch x num_others serialized programs, row-major; each resolves its qubits
 * with the map of its reference program and must use exactly its qubits
 * (ResolveQubitIds with other_programs, program_resolution.cc:188-310) and
 * hold no symbols.  Replaces the parse part of TfqInnerProductOp::Compute
 * (math_ops/tfq_inner_product.cc:48-166). */
int tfqg_batch_create_inner_product(const char* const* programs,
                                    const int64_t* program_lens, int64_t batch,
                                    const char* const* symbol_names,
                                    const int64_t* symbol_name_lens, int64_t num_symbols,
                                    const char* const* other_programs,
                                    const int64_t* other_program_lens, int64_t num_others,
                                    int with_grads, tfqg_batch** out);

/* <psi_i | phi_ij> as complex64 [batch, num_others] (interleaved re, im),
 * fp64 sums; 1 for an empty reference program.  Replaces
 * TfqInnerProductOp::ComputeLarge/Small (math_ops/tfq_inner_product.cc:
 * 168-279).  symbol_values is [batch, num_symbols] for the reference
 * programs. */
int tfqg_batch_inner_product(tfqg_batch* b, const float* symbol_values,
                             void* inner_products, int device_buffers, void* stream);

/* Gradient of the inner products weighted by downstream_grads float
 * [batch, num_others]: complex64 [batch, num_symbols], grads[i, p] = sum over
 * the gates using symbol p of <dU psi | chi_i>, chi_i = sum_j g_ij |phi_ij>
 * (reference finite-difference gradient gates).  Replaces
 * TfqInnerProductGradOp (math_ops/tfq_inner_product_grad.cc:46-452).  The
 * batch must be created with with_grads = 1. */
int tfqg_batch_inner_product_grad(tfqg_batch* b, const float* symbol_values,
                                  const float* downstream_grads, void* grads,
                                  int device_buffers, void* stream);

/* Noisy sampled expectations [batch, num_ops]: num_samples int32
 * [batch, num_ops] trajectories per entry; in each trajectory every Pauli
 * term is measured once (a +-1 parity drawn with P(+1) = (1 + <P>)/2 from the
 * trajectory's state) and the per-entry mean is returned; -2 for empty
 * programs.  Replaces TfqNoisySampledExpectationOp (noise/
 * tfq_noisy_sampled_expectation.cc:143-404).  TFQG_KIND_NOISY batches. */
int tfqg_batch_noisy_sampled_expectation(tfqg_batch* b, const float* symbol_values,
                                         const int32_t* num_samples, uint64_t seed,
                                         float* expectations, int device_buffers,
                                         void* stream);

/* Noisy samples int8 [batch, num_samples, max_num_qubits]: each sample is
 * the measurement of every qubit at the end of its own trajectory, in the
 * layout of tfqg_batch_samples (-2 padding).  Replaces TfqNoisySamplesOp
 * (noise/tfq_noisy_samples.cc:55-280).  TFQG_KIND_NOISY batches. */
int tfqg_batch_noisy_samples(tfqg_batch* b, const float* symbol_values,
                             int32_t num_samples, uint64_t seed, int8_t* samples,
                             int device_buffers, void* stream);

/* Same result as tfqg_batch_expectation, for callers that must not let the
 * library allocate device memory (for example a host framework whose caching
 * allocator has already reserved nearly all device memory, so a plugin's own
 * cudaMalloc can fail).  This entry point has no counterpart in the reference.
 * symbol_values and expectations are DEVICE pointers; the call is
 * asynchronous on `stream`.  All scratch (compiled tables, gate matrices,
 * state slots) lives in one fixed 64 MiB device array owned by the library:
 * larger batches fail with RESOURCE_EXHAUSTED.  Calls share that array, so
 * calls that overlap on the GPU race; the first call on a device looks up the
 * array's address and should come before any stream capture. */
int tfqg_batch_expectation_noalloc(tfqg_batch* b, const float* symbol_values,
                                   float* expectations, void* stream);

/* ---------------------------------------------------------------------
 * CUDA graphs of a batch's forward calls: one call (0 expectation, 1 state,
 * 2 samples) with DEVICE buffers captured once and replayed per step.  The
 * reference runs each op call as a fresh Compute (ComputeSmall/Large of
 * tfq_simulate_expectation_op.cc:182-250, tfq_simulate_samples_op.cc:191-251);
 * here a whole batched call -- matrix build, the persistent queue kernel,
 * the lockstep and wide-row launches -- becomes one graph launch.
 * tfqg_batch_graph_create runs the call once normally (buffers, tables and
 * compiled modules in place), then captures it on `stream` (not the legacy
 * default stream).  A replay reads the symbol values and writes the output
 * at the captured device pointers, so new values written there are used;
 * samples replay with the captured seed.  A replay is refused (INVALID_ARGUMENT)
 * once another call on the batch has replaced one of its device buffers.
 * The graph must be destroyed before its batch.
 * ------------------------------------------------------------------- */
typedef struct tfqg_graph tfqg_graph;
int tfqg_batch_graph_create(tfqg_batch* b, int what, const float* symbol_values,
                            int32_t num_samples, uint64_t seed, void* out, void* stream,
                            tfqg_graph** graph);
int tfqg_graph_launch(tfqg_graph* g, void* stream);
void tfqg_graph_destroy(tfqg_graph* g);

/* ---------------------------------------------------------------------
 * One-shot entry points with the reference op signatures and HOST buffers
 * (what a TF CPU-side OpKernel::Compute holds).  They create a transient
 * batch, run it and destroy it.
 * ------------------------------------------------------------------- */
/* tfq_simulate_expectation (tfq_simulate_ops.py:22-45) */
int tfqg_simulate_expectation(const char* const* programs,
                              const int64_t* program_lens, int64_t batch,
                              const char* const* symbol_names,
                              const int64_t* symbol_name_lens,
                              int64_t num_symbols, const float* symbol_values,
                              const char* const* pauli_sums,
                              const int64_t* pauli_sum_lens, int64_t num_ops,
                              float* expectations);

/* The largest qubit count among the programs: the output width of the
 * state op (2^max) and of the samples op (max), which the reference's
 * Compute derives from the parsed programs before allocate_output
 * (GetProgramsAndNumQubits, parse_context.cc:268-320; used by
 * tfq_simulate_state_op.cc:79-87 and tfq_simulate_samples_op.cc:76-87). */
int tfqg_max_num_qubits(const char* const* programs, const int64_t* program_lens,
                        int64_t batch, int32_t* max_num_qubits);

/* tfq_simulate_state (tfq_simulate_ops.py:48-70; TfqSimulateStateOp::Compute
 * tfq_simulate_state_op.cc:48-215, registered at :221-242).  states:
 * complex64 [batch, 2^max_num_qubits] as (re, im) float pairs; rows of
 * fewer qubits are padded with -2 (tfq_simulate_state_op.cc:201-207).
 * max_num_qubits must be tfqg_max_num_qubits() of the programs. */
int tfqg_simulate_state(const char* const* programs, const int64_t* program_lens,
                        int64_t batch, const char* const* symbol_names,
                        const int64_t* symbol_name_lens, int64_t num_symbols,
                        const float* symbol_values, int32_t max_num_qubits,
                        void* states);

/* tfq_simulate_samples (tfq_simulate_ops.py:73-98; TfqSimulateSamplesOp::
 * Compute tfq_simulate_samples_op.cc:53-251, registered at :258-285).
 * samples: int8 [batch, num_samples, max_num_qubits]; bit k of a sample in
 * column max_num_qubits-k-1, -2 in the leading columns of smaller rows
 * (tfq_simulate_samples_op.cc:227-243).  num_samples < 0 is
 * INVALID_ARGUMENT; 0 writes nothing (tfq_simulate_samples_op.cc:113).
 * max_num_qubits must be tfqg_max_num_qubits() of the programs. */
int tfqg_simulate_samples(const char* const* programs, const int64_t* program_lens,
                          int64_t batch, const char* const* symbol_names,
                          const int64_t* symbol_name_lens, int64_t num_symbols,
                          const float* symbol_values, int32_t num_samples, uint64_t seed,
                          int32_t max_num_qubits, int8_t* samples);

/* tfq_adj_grad (tfq_adj_grad_op.py:22-48) */
int tfqg_adj_grad(const char* const* programs, const int64_t* program_lens,
                  int64_t batch, const char* const* symbol_names,
                  const int64_t* symbol_name_lens, int64_t num_symbols,
                  const float* symbol_values, const char* const* pauli_sums,
                  const int64_t* pauli_sum_lens, int64_t num_ops,
                  const float* downstream_grads, float* grads);

/* tfq.noise.expectation (noise/noisy_expectation_op.py:23-98) */
int tfqg_noisy_expectation(const char* const* programs,
                           const int64_t* program_lens, int64_t batch,
                           const char* const* symbol_names,
                           const int64_t* symbol_name_lens,
                           int64_t num_symbols, const float* symbol_values,
                           const char* const* pauli_sums,
                           const int64_t* pauli_sum_lens, int64_t num_ops,
                           const int32_t* num_samples, uint64_t seed,
                           float* expectations);

/* tfq_simulate_sampled_expectation (tfq_simulate_ops.py:101-135) */
int tfqg_simulate_sampled_expectation(const char* const* programs,
                                      const int64_t* program_lens, int64_t batch,
                                      const char* const* symbol_names,
                                      const int64_t* symbol_name_lens,
                                      int64_t num_symbols, const float* symbol_values,
                                      const char* const* pauli_sums,
                                      const int64_t* pauli_sum_lens, int64_t num_ops,
                                      const int32_t* num_samples, uint64_t seed,
                                      float* expectations);

/* tfq.noise.sampled_expectation (noise/noisy_sampled_expectation_op.py) */
int tfqg_noisy_sampled_expectation(const char* const* programs,
                                   const int64_t* program_lens, int64_t batch,
                                   const char* const* symbol_names,
                                   const int64_t* symbol_name_lens, int64_t num_symbols,
                                   const float* symbol_values,
                                   const char* const* pauli_sums,
                                   const int64_t* pauli_sum_lens, int64_t num_ops,
                                   const int32_t* num_samples, uint64_t seed,
                                   float* expectations);

/* tfq.noise.samples (noise/noisy_samples_op.py) */
int tfqg_noisy_samples(const char* const* programs, const int64_t* program_lens,
                       int64_t batch, const char* const* symbol_names,
                       const int64_t* symbol_name_lens, int64_t num_symbols,
                       const float* symbol_values, int32_t num_samples, uint64_t seed,
                       int8_t* samples);

/* tfq_inner_product (math_ops/inner_product_op.py) */
int tfqg_inner_product(const char* const* programs, const int64_t* program_lens,
                       int64_t batch, const char* const* symbol_names,
                       const int64_t* symbol_name_lens, int64_t num_symbols,
                       const float* symbol_values, const char* const* other_programs,
                       const int64_t* other_program_lens, int64_t num_others,
                       void* inner_products);

#ifdef __cplusplus
}
#endif

#endif /* TFQ_GB300_H_ */
