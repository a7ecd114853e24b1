"""torch.autograd binding: forward = tfq_simulate_expectation, backward =
tfq_adj_grad with the incoming gradient as `downstream_grads`.

This is the torch counterpart of the reference's differentiable expectation
op (tensorflow_quantum/python/differentiators/differentiator.py:153-187 wraps
the forward op with tf.custom_gradient; the Adjoint differentiator
tensorflow_quantum/python/differentiators/adjoint.py:98-103 calls
tfq_adj_grad(programs, symbol_names, symbol_values, pauli_sums, grad)).
"""

import torch

from .ops import Batch, GRAD_REFERENCE_FD, KIND_ADJOINT


class _ExpectationFn(torch.autograd.Function):

    @staticmethod
    def forward(ctx, symbol_values, batch, grad_rule):
        ctx.batch = batch
        ctx.grad_rule = grad_rule
        ctx.save_for_backward(symbol_values)
        return batch.expectation(symbol_values)

    @staticmethod
    def backward(ctx, grad_output):
        (values,) = ctx.saved_tensors
        grads = ctx.batch.adj_grad(values, grad_output.contiguous(),
                                   ctx.grad_rule)
        return grads.to(values.dtype), None, None


class Expectation:
    """Differentiable expectation of fixed circuits and observables.

    >>> layer = Expectation(programs, symbol_names, pauli_sums)
    >>> e = layer(values)            # values: [batch, num_symbols] CUDA tensor
    >>> e.sum().backward()           # adjoint gradient into values.grad
    """

    def __init__(self, programs, symbol_names, pauli_sums,
                 grad_rule=GRAD_REFERENCE_FD):
        self.batch = Batch(programs, symbol_names, pauli_sums, KIND_ADJOINT)
        self.grad_rule = grad_rule

    def __call__(self, symbol_values):
        return _ExpectationFn.apply(symbol_values, self.batch, self.grad_rule)


def expectation(programs, symbol_names, symbol_values, pauli_sums,
                grad_rule=GRAD_REFERENCE_FD):
    """One-shot differentiable expectation."""
    return Expectation(programs, symbol_names, pauli_sums, grad_rule)(
        symbol_values)
