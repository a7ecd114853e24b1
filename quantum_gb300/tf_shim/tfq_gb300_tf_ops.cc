// TensorFlow custom ops over the tfq_gb300 C ABI: the five state-vector ops of
// TensorFlow Quantum registered under their reference names, so that
// tfq.layers, tfq.differentiators and the reference's Python wrappers run on
// this library once this file's .so is loaded in place of the reference's
// _tfq_simulate_ops.so / _tfq_adj_grad.so / noise/_tfq_noise_ops.so.
//
//   op                     reference registration (inputs, outputs, shapes)
//   TfqSimulateExpectation tfq_simulate_expectation_op.cc:257-283
//   TfqSimulateState       tfq_simulate_state_op.cc:221-242
//   TfqSimulateSamples     tfq_simulate_samples_op.cc:258-285
//   TfqAdjointGradient     tfq_adj_grad_op.cc:397-427
//   TfqNoisyExpectation    noise/tfq_noisy_expectation.cc:398-428
//
// Each Compute parses its string tensors into a tfqg_batch (the ABI's
// compiled batch), allocates the output the reference allocates and runs the
// batch on the GPU.  The kernels are registered for DEVICE_CPU: TF hands them
// host tensors, the library copies inputs to the GPU and results back.
// Errors come back as TF status codes with the reference's message texts.
//
// Built by build.py next to this file, only where TensorFlow's headers are
// installed; the repository's tests compile it against the small stand-in
// headers in stub/ to keep it syntactically in step with the ABI.
#include <cstdint>
#include <string>
#include <vector>

#include "tensorflow/core/framework/op.h"
#include "tensorflow/core/framework/op_kernel.h"
#include "tensorflow/core/framework/shape_inference.h"
#include "tensorflow/core/lib/random/random.h"
#include "tfq_gb300.h"

namespace tfq_gb300_tf {

using tensorflow::OpKernel;
using tensorflow::OpKernelConstruction;
using tensorflow::OpKernelContext;
using tensorflow::Status;
using tensorflow::Tensor;
using tensorflow::shape_inference::DimensionHandle;
using tensorflow::shape_inference::InferenceContext;
using tensorflow::shape_inference::ShapeHandle;

// A string tensor as the ABI's (pointer, length) arrays; the views borrow
// the tensor's tstring storage for the duration of Compute.
class StringViews {
 public:
  explicit StringViews(const Tensor& t) {
    auto flat = t.flat<tensorflow::tstring>();
    ptr_.reserve(flat.size());
    len_.reserve(flat.size());
    for (int64_t i = 0; i < flat.size(); ++i) {
      ptr_.push_back(flat(i).data());
      len_.push_back(static_cast<int64_t>(flat(i).size()));
    }
  }
  const char* const* ptr() const { return ptr_.data(); }
  const int64_t* len() const { return len_.data(); }

 private:
  std::vector<const char*> ptr_;
  std::vector<int64_t> len_;
};

// ABI return code -> TF status (the ABI's codes are TF's error codes).
Status FromCode(int rc) {
  if (rc == TFQG_OK) return Status();
  return Status(static_cast<absl::StatusCode>(rc), tfqg_last_error());
}

// Owns a batch for the duration of one Compute.
struct BatchGuard {
  tfqg_batch* b = nullptr;
  ~BatchGuard() {
    if (b) tfqg_batch_destroy(b);
  }
};

// Shape function: every input checked against its rank, the output built
// from input dimensions (input index, dimension) or unknown (-1, -1).
struct DimRef {
  int input, dim;
};

Status CheckRanks(InferenceContext* c, std::initializer_list<int> ranks,
                  std::vector<ShapeHandle>* shapes) {
  int i = 0;
  for (const int r : ranks) {
    ShapeHandle h;
    TF_RETURN_IF_ERROR(c->WithRank(c->input(i), r, &h));
    shapes->push_back(h);
    ++i;
  }
  return Status();
}

Status OutputFrom(InferenceContext* c, const std::vector<ShapeHandle>& in,
                  std::initializer_list<DimRef> dims) {
  std::vector<DimensionHandle> out;
  for (const DimRef& d : dims)
    out.push_back(d.input < 0 ? c->UnknownDim() : c->Dim(in[d.input], d.dim));
  c->set_output(0, c->MakeShape(out));
  return Status();
}

// Inputs shared by all five ops: programs [B], symbol_names [P],
// symbol_values [B, P].
struct Common {
  const Tensor* programs;
  const Tensor* names;
  const Tensor* values;
  int64_t batch() const { return programs->dim_size(0); }
  int64_t symbols() const { return names->dim_size(0); }
};

Common GetCommon(OpKernelContext* ctx) {
  return Common{&ctx->input(0), &ctx->input(1), &ctx->input(2)};
}

Status CreateBatch(const Common& in, const Tensor* pauli_sums, int kind, BatchGuard* g) {
  StringViews p(*in.programs), n(*in.names);
  if (pauli_sums) {
    StringViews s(*pauli_sums);
    return FromCode(tfqg_batch_create(p.ptr(), p.len(), in.batch(), n.ptr(), n.len(),
                                      in.symbols(), s.ptr(), s.len(), pauli_sums->dim_size(1),
                                      kind, &g->b));
  }
  return FromCode(tfqg_batch_create(p.ptr(), p.len(), in.batch(), n.ptr(), n.len(),
                                    in.symbols(), nullptr, nullptr, 0, kind, &g->b));
}

class SimulateExpectation : public OpKernel {
 public:
  explicit SimulateExpectation(OpKernelConstruction* c) : OpKernel(c) {}
  void Compute(OpKernelContext* ctx) override {
    const Common in = GetCommon(ctx);
    const Tensor& psums = ctx->input(3);
    OP_REQUIRES(ctx, psums.dims() == 2,
                tensorflow::errors::InvalidArgument("pauli_sums must be rank 2. Got rank ",
                                                    psums.dims(), "."));
    Tensor* out = nullptr;
    OP_REQUIRES_OK(ctx, ctx->allocate_output(
                            0, tensorflow::TensorShape({in.batch(), psums.dim_size(1)}),
                            &out));
    BatchGuard g;
    OP_REQUIRES_OK(ctx, CreateBatch(in, &psums, TFQG_KIND_FORWARD, &g));
    OP_REQUIRES_OK(ctx, FromCode(tfqg_batch_expectation(g.b, in.values->flat<float>().data(),
                                                         out->flat<float>().data(), 0,
                                                         nullptr)));
  }
};

class SimulateState : public OpKernel {
 public:
  explicit SimulateState(OpKernelConstruction* c) : OpKernel(c) {}
  void Compute(OpKernelContext* ctx) override {
    const Common in = GetCommon(ctx);
    BatchGuard g;
    OP_REQUIRES_OK(ctx, CreateBatch(in, nullptr, TFQG_KIND_FORWARD, &g));
    int32_t max_n = 0;
    OP_REQUIRES_OK(ctx, FromCode(tfqg_batch_max_num_qubits(g.b, &max_n)));
    Tensor* out = nullptr;
    OP_REQUIRES_OK(ctx, ctx->allocate_output(
                            0, tensorflow::TensorShape({in.batch(), int64_t(1) << max_n}),
                            &out));
    OP_REQUIRES_OK(ctx,
                   FromCode(tfqg_batch_state(g.b, in.values->flat<float>().data(),
                                             out->flat<tensorflow::complex64>().data(), 0,
                                             nullptr)));
  }
};

class SimulateSamples : public OpKernel {
 public:
  explicit SimulateSamples(OpKernelConstruction* c) : OpKernel(c) {}
  void Compute(OpKernelContext* ctx) override {
    const Common in = GetCommon(ctx);
    const Tensor& ns = ctx->input(3);
    OP_REQUIRES(ctx, ns.dims() == 1 && ns.dim_size(0) == 1,
                tensorflow::errors::InvalidArgument(
                    "num_samples must contain exactly one value."));
    const int32_t num_samples = ns.flat<int32_t>()(0);
    BatchGuard g;
    OP_REQUIRES_OK(ctx, CreateBatch(in, nullptr, TFQG_KIND_FORWARD, &g));
    int32_t max_n = 0;
    OP_REQUIRES_OK(ctx, FromCode(tfqg_batch_max_num_qubits(g.b, &max_n)));
    Tensor* out = nullptr;
    OP_REQUIRES_OK(ctx, ctx->allocate_output(
                            0, tensorflow::TensorShape({in.batch(), num_samples, max_n}),
                            &out));
    // fresh seed per call, as the reference seeds each call anew
    const uint64_t seed = tensorflow::random::New64();
    OP_REQUIRES_OK(ctx, FromCode(tfqg_batch_samples(g.b, in.values->flat<float>().data(),
                                                     num_samples, seed,
                                                     out->flat<int8_t>().data(), 0, nullptr)));
  }
};

class AdjointGradient : public OpKernel {
 public:
  explicit AdjointGradient(OpKernelConstruction* c) : OpKernel(c) {}
  void Compute(OpKernelContext* ctx) override {
    const Common in = GetCommon(ctx);
    const Tensor& psums = ctx->input(3);
    const Tensor& dgrads = ctx->input(4);
    OP_REQUIRES(ctx, psums.dims() == 2,
                tensorflow::errors::InvalidArgument("pauli_sums must be rank 2. Got rank ",
                                                    psums.dims(), "."));
    Tensor* out = nullptr;
    OP_REQUIRES_OK(ctx, ctx->allocate_output(
                            0, tensorflow::TensorShape({in.batch(), in.symbols()}), &out));
    BatchGuard g;
    OP_REQUIRES_OK(ctx, CreateBatch(in, &psums, TFQG_KIND_ADJOINT, &g));
    OP_REQUIRES_OK(ctx, FromCode(tfqg_batch_adj_grad(
                            g.b, in.values->flat<float>().data(),
                            dgrads.flat<float>().data(), TFQG_GRAD_REFERENCE_FD,
                            out->flat<float>().data(), 0, nullptr)));
  }
};

class NoisyExpectation : public OpKernel {
 public:
  explicit NoisyExpectation(OpKernelConstruction* c) : OpKernel(c) {}
  void Compute(OpKernelContext* ctx) override {
    const Common in = GetCommon(ctx);
    const Tensor& psums = ctx->input(3);
    const Tensor& reps = ctx->input(4);
    OP_REQUIRES(ctx, psums.dims() == 2,
                tensorflow::errors::InvalidArgument("pauli_sums must be rank 2. Got rank ",
                                                    psums.dims(), "."));
    Tensor* out = nullptr;
    OP_REQUIRES_OK(ctx, ctx->allocate_output(
                            0, tensorflow::TensorShape({in.batch(), psums.dim_size(1)}),
                            &out));
    BatchGuard g;
    OP_REQUIRES_OK(ctx, CreateBatch(in, &psums, TFQG_KIND_NOISY, &g));
    const uint64_t seed = tensorflow::random::New64();
    OP_REQUIRES_OK(ctx, FromCode(tfqg_batch_noisy_expectation(
                            g.b, in.values->flat<float>().data(),
                            reps.flat<int32_t>().data(), seed, out->flat<float>().data(), 0,
                            nullptr)));
  }
};

}  // namespace tfq_gb300_tf

using tfq_gb300_tf::CheckRanks;
using tfq_gb300_tf::OutputFrom;

// Shape functions: the reference's rank checks; outputs [B, ops],
// [B, unknown], [B, unknown, unknown], [B, P], [B, ops].
REGISTER_OP("TfqSimulateExpectation")
    .Input("programs: string")
    .Input("symbol_names: string")
    .Input("symbol_values: float")
    .Input("pauli_sums: string")
    .Output("expectations: float")
    .SetShapeFn([](tensorflow::shape_inference::InferenceContext* c) {
      std::vector<tensorflow::shape_inference::ShapeHandle> in;
      TF_RETURN_IF_ERROR(CheckRanks(c, {1, 1, 2, 2}, &in));
      return OutputFrom(c, in, {{0, 0}, {3, 1}});
    });

REGISTER_OP("TfqSimulateState")
    .Input("programs: string")
    .Input("symbol_names: string")
    .Input("symbol_values: float")
    .Output("state_vector: complex64")
    .SetShapeFn([](tensorflow::shape_inference::InferenceContext* c) {
      std::vector<tensorflow::shape_inference::ShapeHandle> in;
      TF_RETURN_IF_ERROR(CheckRanks(c, {1, 1, 2}, &in));
      return OutputFrom(c, in, {{0, 0}, {-1, -1}});
    });

REGISTER_OP("TfqSimulateSamples")
    .Input("programs: string")
    .Input("symbol_names: string")
    .Input("symbol_values: float")
    .Input("num_samples: int32")
    .Output("samples: int8")
    .SetShapeFn([](tensorflow::shape_inference::InferenceContext* c) {
      std::vector<tensorflow::shape_inference::ShapeHandle> in;
      TF_RETURN_IF_ERROR(CheckRanks(c, {1, 1, 2, 1}, &in));
      return OutputFrom(c, in, {{0, 0}, {-1, -1}, {-1, -1}});
    });

REGISTER_OP("TfqAdjointGradient")
    .Input("programs: string")
    .Input("symbol_names: string")
    .Input("symbol_values: float")
    .Input("pauli_sums: string")
    .Input("downstream_grads: float")
    .Output("grads: float")
    .SetShapeFn([](tensorflow::shape_inference::InferenceContext* c) {
      std::vector<tensorflow::shape_inference::ShapeHandle> in;
      TF_RETURN_IF_ERROR(CheckRanks(c, {1, 1, 2, 2, 2}, &in));
      return OutputFrom(c, in, {{0, 0}, {1, 0}});
    });

REGISTER_OP("TfqNoisyExpectation")
    .Input("programs: string")
    .Input("symbol_names: string")
    .Input("symbol_values: float")
    .Input("pauli_sums: string")
    .Input("num_samples: int32")
    .Output("expectations: float")
    .SetShapeFn([](tensorflow::shape_inference::InferenceContext* c) {
      std::vector<tensorflow::shape_inference::ShapeHandle> in;
      TF_RETURN_IF_ERROR(CheckRanks(c, {1, 1, 2, 2, 2}, &in));
      return OutputFrom(c, in, {{0, 0}, {3, 1}});
    });

REGISTER_KERNEL_BUILDER(Name("TfqSimulateExpectation").Device(tensorflow::DEVICE_CPU),
                        tfq_gb300_tf::SimulateExpectation);
REGISTER_KERNEL_BUILDER(Name("TfqSimulateState").Device(tensorflow::DEVICE_CPU),
                        tfq_gb300_tf::SimulateState);
REGISTER_KERNEL_BUILDER(Name("TfqSimulateSamples").Device(tensorflow::DEVICE_CPU),
                        tfq_gb300_tf::SimulateSamples);
REGISTER_KERNEL_BUILDER(Name("TfqAdjointGradient").Device(tensorflow::DEVICE_CPU),
                        tfq_gb300_tf::AdjointGradient);
REGISTER_KERNEL_BUILDER(Name("TfqNoisyExpectation").Device(tensorflow::DEVICE_CPU),
                        tfq_gb300_tf::NoisyExpectation);
