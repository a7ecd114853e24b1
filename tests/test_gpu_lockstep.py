"""Lockstep rows (forward modes): streamed rows of 17-21 qubits that are not
wide run side by side over the whole grid, one launch per pass index (tile
passes) or per block index (5-qubit tensor-core blocks), instead of one CTA
each.  Expectation (and the per-term values of the sampled expectation),
state with padding, and samples against the oracle, with the rows split
over several lockstep groups, under both gate paths, and against the same
batch run through the queue (lockstep off)."""

import numpy as np
import pytest

from oracle import tfq_oracle as O
from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S
from tests.circuits import expectation_atol, random_circuit, random_paulisum
from tests.stats import bits_to_index, chi2_pvalue

pytestmark = pytest.mark.gpu

NQS = [17, 6, 18, 17, 14, 19, 17, 10]


@pytest.fixture(params=[False, True], ids=["tile_passes", "tensor_cores"])
def lockstep(request):
    """Lockstep from 17 qubits, no few-rows wide rule, small groups (three
    groups over the batch's five lock rows); the rows' gates on tile passes
    or on tensor-core blocks."""
    old = (_native.set_lock_min_qubits(17), _native.set_wide_few_rows(0),
           _native.set_lock_arena_amps(1 << 19), _native.set_lock_tc(request.param))
    yield request.param
    _native.set_lock_min_qubits(old[0])
    _native.set_wide_few_rows(old[1])
    _native.set_lock_arena_amps(old[2])
    _native.set_lock_tc(old[3])


def _check_path(b, tc):
    blocks, units = _native.batch_lock_tc(b._h)
    if tc:
        assert blocks > 0 and units >= blocks, (blocks, units)
    else:
        assert blocks == 0 and units == 0, (blocks, units)


def _inputs(seed):
    rng = np.random.default_rng(seed)
    names = ["a", "b", "c"]
    programs, psums = [], []
    for n in NQS:
        qs = S.GridQubit.rect(1, n)
        programs.append(S.serialize_circuit(random_circuit(qs, 4, rng, names, p_control=0.2)))
        psums.append([random_paulisum(qs, rng) for _ in range(2)])
    values = rng.uniform(-2, 2, size=(len(NQS), 3)).astype(np.float32)
    return programs, names, values, psums


def test_expectation_and_state(lockstep):
    programs, names, values, psums = _inputs(1)
    b = ops.Batch(programs, names, psums)
    rows, groups = _native.batch_lock_rows(b._h)
    assert rows == 5 and groups >= 3, (rows, groups)
    _check_path(b, lockstep)
    got = b.expectation(values)
    want = O.simulate_expectation(programs, names, values, psums)
    np.testing.assert_allclose(got, want, atol=expectation_atol(psums), rtol=0)
    sb = ops.Batch(programs, names, None)
    _check_path(sb, lockstep)
    st = sb.state(values)
    np.testing.assert_allclose(st, O.simulate_state(programs, names, values), atol=1e-5, rtol=0)
    # the same batch through the queue, one CTA per row
    _native.set_lock_min_qubits(99)
    q = ops.Batch(programs, names, psums)
    assert _native.batch_lock_rows(q._h)[0] == 0
    np.testing.assert_allclose(got, q.expectation(values), atol=1e-6, rtol=0)


def test_sampled_expectation_term_values(lockstep):
    programs, names, values, psums = _inputs(2)
    b = ops.Batch(programs, names, psums)
    assert _native.batch_lock_rows(b._h)[0] == 5
    _check_path(b, lockstep)
    R = 40000
    got = b.sampled_expectation(values, np.full((len(NQS), 2), R, np.int32), seed=5)
    want = O.simulate_expectation(programs, names, values, psums)
    bound = 5 * expectation_atol(psums, 1.0) / np.sqrt(R)
    np.testing.assert_allclose(got, want, atol=bound, rtol=0)


def test_samples(lockstep):
    programs, names, values, _ = _inputs(3)
    b = ops.Batch(programs, names, None)
    assert _native.batch_lock_rows(b._h)[0] == 5
    _check_path(b, lockstep)
    shots = 4000
    s = b.samples(values, shots, seed=9)
    maxn = max(NQS)
    probs = O.final_probabilities(programs, names, values)
    for r, n in enumerate(NQS):
        assert (s[r, :, :maxn - n] == -2).all()
        if n >= 17:
            counts = np.bincount(bits_to_index(s[r], n), minlength=2 ** n)
            p, chi2, bins = chi2_pvalue(counts, probs[r][1], shots)
            assert p > 1e-3, (r, n, chi2, bins, p)


def test_repeated_program_rows(lockstep):
    """Rows with one program and one observable list (a batch of symbol
    values for the same circuit) share their measurement passes; every row
    still keeps its own term sums, in every lockstep group."""
    rng = np.random.default_rng(4)
    names = ["a", "b", "c"]
    qs = S.GridQubit.rect(1, 17)
    prog = S.serialize_circuit(random_circuit(qs, 4, rng, names, p_control=0.2))
    ps = [random_paulisum(qs, rng) for _ in range(2)]
    programs, psums = [prog] * 6, [ps] * 6
    values = rng.uniform(-2, 2, size=(6, 3)).astype(np.float32)
    b = ops.Batch(programs, names, psums)
    rows, groups = _native.batch_lock_rows(b._h)
    assert rows == 6 and groups >= 2, (rows, groups)
    _check_path(b, lockstep)
    got = b.expectation(values)
    want = O.simulate_expectation(programs, names, values, psums)
    assert np.ptp(want[:, 0]) > 1e-3  # the rows differ
    np.testing.assert_allclose(got, want, atol=expectation_atol(psums), rtol=0)
    R = 40000
    got = b.sampled_expectation(values, np.full((6, 2), R, np.int32), seed=3)
    bound = 5 * expectation_atol(psums, 1.0) / np.sqrt(R)
    np.testing.assert_allclose(got, want, atol=bound, rtol=0)
