// Stand-in declarations of TensorFlow's shape-inference API (syntax check
// of tfq_gb300_tf_ops.cc only; nothing here is linked or run).
#pragma once
#include <vector>

#include "tensorflow/core/framework/op_kernel.h"

namespace tensorflow {
namespace shape_inference {

class ShapeHandle {};
class DimensionHandle {};

class InferenceContext {
 public:
  ShapeHandle input(int i) const;
  Status WithRank(ShapeHandle s, int rank, ShapeHandle* out);
  DimensionHandle Dim(ShapeHandle s, int d);
  DimensionHandle UnknownDim();
  ShapeHandle MakeShape(const std::vector<DimensionHandle>& dims);
  void set_output(int i, ShapeHandle s);
};

}  // namespace shape_inference
}  // namespace tensorflow

#define TF_RETURN_IF_ERROR(...)                 \
  do {                                          \
    ::tensorflow::Status _st(__VA_ARGS__);      \
    if (!_st.ok()) return _st;                  \
  } while (0)
