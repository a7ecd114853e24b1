// Stand-in declarations of the TensorFlow op-kernel API used by
// tfq_gb300_tf_ops.cc, for a syntax check where TensorFlow is not installed.
// Declarations only: nothing here is linked or run.
#pragma once
#include <complex>
#include <cstdint>
#include <initializer_list>
#include <string>

namespace absl {
enum class StatusCode : int {};
}

namespace tensorflow {

class Status {
 public:
  Status();
  Status(absl::StatusCode code, const char* msg);
  bool ok() const;
};

using complex64 = std::complex<float>;

class tstring {
 public:
  const char* data() const;
  size_t size() const;
};

template <class T>
class TTypesFlat {
 public:
  int64_t size() const;
  const T& operator()(int64_t i) const;
  T& operator()(int64_t i);
  T* data();
  const T* data() const;
};

class TensorShape {
 public:
  TensorShape(std::initializer_list<int64_t> dims);
};

class Tensor {
 public:
  int dims() const;
  int64_t dim_size(int d) const;
  template <class T>
  TTypesFlat<T> flat() const;
};

class OpKernelConstruction {};

class OpKernelContext {
 public:
  const Tensor& input(int i);
  Status allocate_output(int i, const TensorShape& shape, Tensor** out);
  void CtxFailure(const char* file, int line, const Status& s);
};

class OpKernel {
 public:
  explicit OpKernel(OpKernelConstruction* c);
  virtual ~OpKernel();
  virtual void Compute(OpKernelContext* ctx) = 0;
};

namespace errors {
template <class... Args>
Status InvalidArgument(Args... args);
}

constexpr const char* DEVICE_CPU = "CPU";

class KernelDefBuilder {
 public:
  KernelDefBuilder& Device(const char* d);
};
KernelDefBuilder Name(const char* op);

namespace register_kernel {
template <class K>
struct Registrar {
  explicit Registrar(const KernelDefBuilder& b);
};
}  // namespace register_kernel

}  // namespace tensorflow

#define OP_REQUIRES(CTX, EXP, STATUS)              \
  do {                                             \
    if (!(EXP)) {                                  \
      (CTX)->CtxFailure(__FILE__, __LINE__, (STATUS)); \
      return;                                      \
    }                                              \
  } while (0)

#define OP_REQUIRES_OK(CTX, ...)                   \
  do {                                             \
    ::tensorflow::Status _s(__VA_ARGS__);          \
    if (!_s.ok()) {                                \
      (CTX)->CtxFailure(__FILE__, __LINE__, _s);   \
      return;                                      \
    }                                              \
  } while (0)

#define TFQG_STUB_CAT2(a, b) a##b
#define TFQG_STUB_CAT(a, b) TFQG_STUB_CAT2(a, b)
#define REGISTER_KERNEL_BUILDER(BUILDER, KERNEL)                                     \
  static ::tensorflow::register_kernel::Registrar<KERNEL> TFQG_STUB_CAT(             \
      tfqg_stub_kernel_, __COUNTER__)(::tensorflow::BUILDER)
