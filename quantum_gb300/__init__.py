"""GB300-native (sm_103a) implementation of TensorFlow Quantum's
state-vector ops: tfq_simulate_expectation / _state / _samples /
_sampled_expectation, tfq_adj_grad, noise.expectation and
math.inner_product, behind a C ABI (include/tfq_gb300.h)."""

from ._native import (InvalidArgumentError, NativeLibraryMissing,  # noqa: F401
                      ResourceExhaustedError, UnimplementedError)
from .ops import (Batch, GRAD_EXACT, GRAD_REFERENCE_FD, InnerProductBatch,  # noqa: F401
                  KIND_ADJOINT, KIND_FORWARD, KIND_INNER, KIND_NOISY,
                  inner_product_grad, noisy_expectation, noisy_sampled_expectation,
                  noisy_samples, tfq_adj_grad,
                  tfq_inner_product,
                  tfq_simulate_expectation, tfq_simulate_sampled_expectation,
                  tfq_simulate_samples, tfq_simulate_state)

__version__ = "0.1.0"
