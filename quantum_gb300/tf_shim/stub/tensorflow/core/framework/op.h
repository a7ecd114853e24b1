// Stand-in declarations of TensorFlow's op registry (syntax check of
// tfq_gb300_tf_ops.cc only; nothing here is linked or run).
#pragma once
#include "tensorflow/core/framework/shape_inference.h"

namespace tensorflow {

class OpDefBuilder {
 public:
  explicit OpDefBuilder(const char* name);
  OpDefBuilder& Input(const char* spec);
  OpDefBuilder& Output(const char* spec);
  OpDefBuilder& SetShapeFn(Status (*fn)(shape_inference::InferenceContext*));
};

struct OpDefReceiver {
  OpDefReceiver(const OpDefBuilder& b);  // NOLINT: implicit, as the macro needs
};

}  // namespace tensorflow

#define TFQG_STUB_OP_CAT2(a, b) a##b
#define TFQG_STUB_OP_CAT(a, b) TFQG_STUB_OP_CAT2(a, b)
#define REGISTER_OP(NAME)                                                       \
  static ::tensorflow::OpDefReceiver TFQG_STUB_OP_CAT(tfqg_stub_op_, __COUNTER__) = \
      ::tensorflow::OpDefBuilder(NAME)
