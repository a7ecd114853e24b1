"""Run-time specialized kernels (NVRTC, one module per batch and mode)
against the complex128 oracle and against the precompiled interpreter on
the same inputs.  Specialization is forced on one handle and off on the
other; the test fails if the specialized module did not load, so a silent
fall back to the interpreter cannot pass.  Tolerances as in
test_gpu_parity.py."""

import numpy as np
import pytest

from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S
from oracle import tfq_oracle as O
from tests.circuits import (CHANNELS, expectation_atol, gradient_atol, random_circuit,
                            random_paulisum)

pytestmark = pytest.mark.gpu


def _inputs(rng, nqs, n_moments=6, n_symbols=5, n_ops=2, channels=()):
    names = [f"s{i}" for i in range(n_symbols)]
    programs, psums = [], []
    for n in nqs:
        qs = S.GridQubit.rect(1, n)
        c = random_circuit(qs, n_moments, rng, names, p_control=0.3,
                           channels=list(channels),
                           p_channel=0.3 if channels else 0.0)
        programs.append(S.serialize_circuit(c))
        psums.append([random_paulisum(qs, rng) for _ in range(n_ops)])
    values = rng.uniform(-2, 2, size=(len(nqs), n_symbols)).astype(np.float32)
    return programs, names, values, psums


def _pair(programs, names, psums, kind):
    """(specialized, interpreter) handles of the same batch."""
    jit = ops.Batch(programs, names, psums, kind=kind)
    ref = ops.Batch(programs, names, psums, kind=kind)
    _native.batch_specialization(jit._h, 1)
    _native.batch_specialization(ref._h, -1)
    return jit, ref


def _assert_loaded(b, mode):
    _, active, err = _native.batch_specialization(b._h)
    assert mode in active, err


@pytest.mark.parametrize("nqs", [[3, 5, 8], [12, 14], [15, 16], [17]])
def test_expectation(nqs):
    rng = np.random.default_rng(40 + sum(nqs))
    programs, names, values, psums = _inputs(rng, nqs)
    jit, ref = _pair(programs, names, psums, ops.KIND_FORWARD)
    got = jit.expectation(values)
    # a lone row of 17+ qubits runs as a wide row (the whole grid on it)
    _assert_loaded(jit, "wide" if min(nqs) >= 17 else "expect")
    want = O.simulate_expectation(programs, names, values, psums)
    np.testing.assert_allclose(got, want, atol=expectation_atol(psums), rtol=0)
    np.testing.assert_allclose(got, ref.expectation(values), atol=1e-6, rtol=0)


@pytest.mark.parametrize("nqs,rule", [([4, 6, 9], 0), ([13, 11], 1),
                                      ([14], 0), ([15, 7], 1)])
def test_adj_grad(nqs, rule):
    rng = np.random.default_rng(70 + sum(nqs) + rule)
    programs, names, values, psums = _inputs(rng, nqs, n_moments=5)
    dg = rng.normal(size=(len(nqs), 2)).astype(np.float32)
    jit, ref = _pair(programs, names, psums, ops.KIND_ADJOINT)
    got = jit.adj_grad(values, dg, grad_rule=rule)
    _assert_loaded(jit, "adjoint")
    want = O.adj_grad(programs, names, values, psums, dg,
                      grad_rule="fd" if rule == 0 else "analytic")
    np.testing.assert_allclose(got, want, atol=gradient_atol(psums, dg), rtol=0)
    np.testing.assert_allclose(got, ref.adj_grad(values, dg, grad_rule=rule),
                               atol=gradient_atol(psums, dg), rtol=0)


@pytest.mark.parametrize("nqs", [[2, 6], [14, 3], [15]])
def test_state(nqs):
    rng = np.random.default_rng(90 + sum(nqs))
    programs, names, values, _ = _inputs(rng, nqs, n_ops=0)
    psums = [[] for _ in nqs]
    jit = ops.Batch(programs, names, None, kind=ops.KIND_FORWARD)
    _native.batch_specialization(jit._h, 1)
    got = jit.state(values)
    _assert_loaded(jit, "state")
    want = O.simulate_state(programs, names, values)
    np.testing.assert_allclose(got, want, atol=1e-5, rtol=0)
    del psums


def test_samples_follow_the_interpreter():
    rng = np.random.default_rng(5)
    programs, names, values, _ = _inputs(rng, [4, 7, 10], n_ops=0)
    jit = ops.Batch(programs, names, None, kind=ops.KIND_FORWARD)
    ref = ops.Batch(programs, names, None, kind=ops.KIND_FORWARD)
    _native.batch_specialization(jit._h, 1)
    _native.batch_specialization(ref._h, -1)
    a = jit.samples(values, 2000, seed=99)
    _assert_loaded(jit, "sample")
    b = ref.samples(values, 2000, seed=99)
    assert a.shape == b.shape
    # same state up to float rounding and the same random stream: draws agree
    # except where a uniform falls within rounding of a CDF boundary
    agree = np.mean(np.all(a == b, axis=2))
    assert agree > 0.99, agree


def test_noisy_expectation():
    rng = np.random.default_rng(21)
    programs, names, values, psums = _inputs(rng, [3, 5], n_moments=5,
                                             channels=CHANNELS)
    jit, ref = _pair(programs, names, psums, ops.KIND_NOISY)
    R = 20000
    reps = np.full((2, 2), R, np.int32)
    got = jit.noisy_expectation(values, reps, seed=3)
    _assert_loaded(jit, "noisy")
    want = O.noisy_expectation_exact(programs, names, values, psums)
    bound = 5 * 8 / np.sqrt(R) + 1e-4
    np.testing.assert_allclose(got, want, atol=bound, rtol=0)
    # same seed: the same branch draws, so the trajectory means agree up to
    # draws that fall within rounding of a branch boundary
    np.testing.assert_allclose(got, ref.noisy_expectation(values, reps, seed=3),
                               atol=2e-3, rtol=0)
