"""Wide rows: states too large for one CTA, simulated by the whole grid one
launch per pass (forward modes and the adjoint gradient: forward, lambda and
backward passes, gradient slots summed across CTAs). The wide threshold is
lowered here so that
15..18-qubit rows take the path at oracle-checkable sizes. Narrow rows of
the same batch still go through the persistent kernel. One 22-qubit row
checks the default threshold. Tolerances as in test_gpu_parity.py."""

import numpy as np
import pytest
from scipy import stats

from oracle import tfq_oracle as O
from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S
from tests.circuits import expectation_atol, gradient_atol, random_circuit, random_paulisum

pytestmark = pytest.mark.gpu


@pytest.fixture
def wide_from_15():
    old = _native.set_wide_min_qubits(15)
    yield
    _native.set_wide_min_qubits(old)


def _inputs(rng, nqs, n_moments=5, n_ops=2, n_symbols=4):
    names = [f"s{i}" for i in range(n_symbols)]
    programs, psums = [], []
    for n in nqs:
        qs = S.GridQubit.rect(1, n)
        programs.append(S.serialize_circuit(random_circuit(qs, n_moments, rng, names,
                                                           p_control=0.3)))
        psums.append([random_paulisum(qs, rng, n_terms=6) for _ in range(n_ops)])
    values = rng.uniform(-2, 2, size=(len(nqs), n_symbols)).astype(np.float32)
    return programs, names, values, psums


@pytest.mark.parametrize("jit", [-1, 1])
def test_expectation_mixed_wide_and_narrow(wide_from_15, jit):
    rng = np.random.default_rng(12 + jit)
    nqs = [16, 5, 17, 15, 12]
    programs, names, values, psums = _inputs(rng, nqs)
    b = ops.Batch(programs, names, psums)
    assert _native.batch_wide_rows(b._h) == 3
    _native.batch_specialization(b._h, jit)
    got = b.expectation(values)
    if jit == 1:
        _, active, err = _native.batch_specialization(b._h)
        assert "wide" in active, err
    want = O.simulate_expectation(programs, names, values, psums)
    np.testing.assert_allclose(got, want, atol=expectation_atol(psums), rtol=0)


def test_adjoint_batch_wide_row_beside_a_queued_row(wide_from_15):
    rng = np.random.default_rng(3)
    programs, names, values, psums = _inputs(rng, [16, 4], n_moments=4)
    b = ops.Batch(programs, names, psums, kind=ops.KIND_ADJOINT)
    assert _native.batch_wide_rows(b._h) == 1
    np.testing.assert_allclose(b.expectation(values),
                               O.simulate_expectation(programs, names, values, psums),
                               atol=expectation_atol(psums), rtol=0)
    dg = rng.normal(size=(2, 2)).astype(np.float32)
    want = O.adj_grad(programs, names, values, psums, dg)
    np.testing.assert_allclose(b.adj_grad(values, dg), want,
                               atol=gradient_atol(psums, dg), rtol=0)


def test_state_with_padding(wide_from_15):
    rng = np.random.default_rng(8)
    programs, names, values, _ = _inputs(rng, [15, 3, 16], n_ops=0)
    b = ops.Batch(programs, names, None)
    assert _native.batch_wide_rows(b._h) == 2
    got = b.state(values)
    want = O.simulate_state(programs, names, values)
    assert got.shape == want.shape == (3, 2 ** 16)
    np.testing.assert_allclose(got, want, atol=1e-5, rtol=0)


def test_samples_distribution_and_layout(wide_from_15):
    q = S.GridQubit.rect(1, 16)
    ops_ = [S.X(q[0]), S.X(q[3]), S.X(q[7]), S.H(q[2]), S.H(q[12])]
    ops_ += [S.I(x) for i, x in enumerate(q) if i not in (0, 2, 3, 7, 12)]
    wide = S.serialize_circuit(S.Circuit([ops_]))
    small = S.serialize_circuit(S.Circuit([[S.X(S.GridQubit(0, 0)), S.I(S.GridQubit(0, 1))]]))
    b = ops.Batch([wide, small], [], None)
    assert _native.batch_wide_rows(b._h) == 1
    shots = 4000
    res = b.samples(np.zeros((2, 0), np.float32), shots, seed=11)
    assert res.shape == (2, shots, 16)
    # narrow row: 2 qubits, 14 leading -2 columns, then bits (q0 = 1, q1 = 0)
    assert (res[1, :, :14] == -2).all()
    assert (res[1, :, 14:] == np.array([1, 0])).all()
    bits = res[0].astype(np.int64)
    idx = (bits[:, ::-1] << np.arange(16)).sum(axis=1)  # column 15 - k holds bit k
    (n, probs), _ = O.final_probabilities([wide, small], [], np.zeros((2, 0)))
    support = np.nonzero(probs > 1e-6)[0]
    assert len(support) == 4 and set(np.unique(idx)) <= set(support)
    counts = np.array([(idx == s).sum() for s in support])
    p = stats.chisquare(counts, probs[support] / probs[support].sum() * shots).pvalue
    assert p > 1e-3, (counts, p)


def test_default_threshold_22_qubits():
    rng = np.random.default_rng(22)
    programs, names, values, psums = _inputs(rng, [22], n_moments=2, n_ops=1)
    b = ops.Batch(programs, names, psums)
    assert _native.batch_wide_rows(b._h) == 1
    np.testing.assert_allclose(b.expectation(values),
                               O.simulate_expectation(programs, names, values, psums),
                               atol=expectation_atol(psums), rtol=0)


@pytest.mark.parametrize("rule", [ops.GRAD_REFERENCE_FD, ops.GRAD_EXACT])
def test_wide_adjoint_gradient_mixed_batch(wide_from_15, rule):
    """Gradients of wide rows (15..17 qubits, symbols shared by several
    gates, controlled gates) beside narrow rows, against the oracle."""
    rng = np.random.default_rng(40 + rule)
    nqs = [16, 5, 15, 17, 9]
    programs, names, values, psums = _inputs(rng, nqs, n_moments=5, n_ops=2)
    b = ops.Batch(programs, names, psums, kind=ops.KIND_ADJOINT)
    assert _native.batch_wide_rows(b._h) == 3
    dg = rng.normal(size=(len(nqs), 2)).astype(np.float32)
    got = b.adj_grad(values, dg, rule)
    want = O.adj_grad(programs, names, values, psums, dg,
                      grad_rule="fd" if rule == ops.GRAD_REFERENCE_FD else "exact")
    np.testing.assert_allclose(got, want, atol=gradient_atol(psums, dg), rtol=0)


def test_wide_adjoint_without_terms_is_zero(wide_from_15):
    """A wide row whose Pauli sums are empty has lambda = 0: zero gradient."""
    rng = np.random.default_rng(5)
    qs = S.GridQubit.rect(1, 16)
    names = ["a", "b"]
    prog = S.serialize_circuit(random_circuit(qs, 4, rng, names, p_control=0.0))
    empty = S.serialize_paulisum([])
    b = ops.Batch([prog], names, [[empty]], kind=ops.KIND_ADJOINT)
    assert _native.batch_wide_rows(b._h) == 1
    got = b.adj_grad(np.array([[0.3, -0.7]], np.float32), np.ones((1, 1), np.float32))
    np.testing.assert_array_equal(got, np.zeros((1, 2), np.float32))


def test_wide_adjoint_default_threshold_22_qubits():
    rng = np.random.default_rng(23)
    programs, names, values, psums = _inputs(rng, [22, 4], n_moments=2, n_ops=1)
    b = ops.Batch(programs, names, psums, kind=ops.KIND_ADJOINT)
    assert _native.batch_wide_rows(b._h) == 1
    dg = np.ones((2, 1), np.float32)
    want = O.adj_grad(programs, names, values, psums, dg)
    np.testing.assert_allclose(b.adj_grad(values, dg), want,
                               atol=gradient_atol(psums, dg), rtol=0)
