// Stand-in declaration of TensorFlow's process-wide random source (syntax
// check of tfq_gb300_tf_ops.cc only).
#pragma once
#include <cstdint>

namespace tensorflow {
namespace random {
uint64_t New64();
}
}  // namespace tensorflow
