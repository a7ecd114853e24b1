"""Lockstep rows on tensor-core blocks: block k of every lockstep row in one
launch (units of up to 16 chunks of one row each, direct and transposed
variants in separate launches), or all blocks of a lockstep group in one
persistent launch whose units wait for their row's earlier blocks.  Rows of 15-19 qubits (streamed rows) against the complex128
oracle and against the same rows on tile passes; a row whose gate spans six
bits (no 5-qubit plan) keeps its tile passes inside a tensor-core group;
deep circuits (many blocks per row, ragged block counts); a timed-out wait
reported by an ordinary call, and marked in the results of a graph replay.
The timeout is injected on the host (or written into the device status word
by the captured call), never caused on the GPU."""

import numpy as np
import pytest

from oracle import tfq_oracle as O
from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S
from tests.circuits import expectation_atol, make_gate, random_circuit, random_paulisum

pytestmark = pytest.mark.gpu

NAMES = ["a", "b", "c"]


@pytest.fixture(params=[True, False], ids=["persistent", "per_block_launches"])
def lock_tc(request):
    """Lockstep from 14 qubits (streamed rows start at 15), no few-rows wide
    rule, groups of at most 2^20 amplitudes, tensor-core blocks on; one
    persistent launch per group or one launch per block index."""
    old = (_native.set_lock_min_qubits(14), _native.set_wide_few_rows(0),
           _native.set_lock_arena_amps(1 << 20), _native.set_lock_tc(True),
           _native.set_tc_lock_persistent(request.param))
    yield
    _native.set_lock_min_qubits(old[0])
    _native.set_wide_few_rows(old[1])
    _native.set_lock_arena_amps(old[2])
    _native.set_lock_tc(old[3])
    _native.set_tc_lock_persistent(old[4])


def _batch(nqs, depths, seed, six_bit_row=None):
    rng = np.random.default_rng(seed)
    programs, psums = [], []
    for r, (n, d) in enumerate(zip(nqs, depths)):
        qs = S.GridQubit.rect(1, n)
        c = random_circuit(qs, d, rng, NAMES, p_control=0.2)
        if r == six_bit_row:
            op = make_gate(rng, "ISP", [qs[1], qs[n - 2]], NAMES, 0.5)
            op = op.controlled_by(qs[0], qs[4], qs[7], qs[n - 1], control_values=[1, 0, 1, 1])
            c.moments.insert(1, [op])
        programs.append(S.serialize_circuit(c))
        psums.append([random_paulisum(qs, rng) for _ in range(2)])
    values = rng.uniform(-2, 2, size=(len(nqs), len(NAMES))).astype(np.float32)
    return programs, values, psums


def _tile_pass_expectation(programs, values, psums):
    old = _native.set_lock_tc(False)
    try:
        q = ops.Batch(programs, NAMES, psums)
        assert _native.batch_lock_tc(q._h) == (0, 0)
        return q.expectation(values)
    finally:
        _native.set_lock_tc(old)


def test_rows_of_15_to_19_qubits(lock_tc):
    nqs = [15, 19, 15, 17, 16, 18, 15, 17]
    programs, values, psums = _batch(nqs, [6] * len(nqs), 11)
    b = ops.Batch(programs, NAMES, psums)
    rows, groups = _native.batch_lock_rows(b._h)
    assert rows == len(nqs) and groups >= 2, (rows, groups)
    blocks, units = _native.batch_lock_tc(b._h)
    assert blocks >= len(nqs) and units > blocks
    got = b.expectation(values)
    want = O.simulate_expectation(programs, NAMES, values, psums)
    np.testing.assert_allclose(got, want, atol=expectation_atol(psums), rtol=0)
    np.testing.assert_allclose(got, _tile_pass_expectation(programs, values, psums),
                               atol=expectation_atol(psums), rtol=0)
    st = ops.Batch(programs, NAMES, None).state(values)
    np.testing.assert_allclose(st, O.simulate_state(programs, NAMES, values), atol=1e-5,
                               rtol=0)


def test_row_without_plan_keeps_tile_passes(lock_tc):
    nqs = [16, 16, 17, 16]
    programs, values, psums = _batch(nqs, [4] * len(nqs), 12, six_bit_row=2)
    b = ops.Batch(programs, NAMES, psums)
    assert _native.batch_lock_rows(b._h)[0] == 4
    blocks, _ = _native.batch_lock_tc(b._h)
    assert blocks > 0
    # the six-bit row has no plan: compare with a batch of the other rows
    others = [0, 1, 3]
    ob = ops.Batch([programs[i] for i in others], NAMES, [psums[i] for i in others])
    assert _native.batch_lock_tc(ob._h)[0] == blocks
    got = b.expectation(values)
    want = O.simulate_expectation(programs, NAMES, values, psums)
    np.testing.assert_allclose(got, want, atol=expectation_atol(psums), rtol=0)


def test_deep_ragged_rows(lock_tc):
    """Rows with 2 to 40 moments: block counts differ per row, so later
    launches cover fewer rows."""
    nqs = [15, 16, 15, 15]
    depths = [40, 2, 25, 9]
    programs, values, psums = _batch(nqs, depths, 13)
    b = ops.Batch(programs, NAMES, psums)
    got = b.expectation(values)
    want = O.simulate_expectation(programs, NAMES, values, psums)
    np.testing.assert_allclose(got, want, atol=expectation_atol(psums), rtol=0)
    st = ops.Batch(programs, NAMES, None).state(values)
    np.testing.assert_allclose(st, O.simulate_state(programs, NAMES, values), atol=2e-5,
                               rtol=0)


def test_timeout_fails_the_call(lock_tc):
    programs, values, psums = _batch([15, 16], [3, 3], 14)
    b = ops.Batch(programs, NAMES, psums)
    assert _native.batch_lock_tc(b._h)[0] > 0
    prev = _native.tc_inject_status(1)
    try:
        with pytest.raises(Exception, match="tensor-core"):
            b.expectation(values)
    finally:
        _native.tc_inject_status(prev)
    want = O.simulate_expectation(programs, NAMES, values, psums)
    np.testing.assert_allclose(b.expectation(values), want, atol=expectation_atol(psums),
                               rtol=0)


def test_graph_replay_marks_a_timeout(lock_tc):
    import torch
    nqs = [15, 9, 16]
    programs, values, psums = _batch(nqs, [3, 3, 3], 15)
    b = ops.Batch(programs, NAMES, psums)
    assert _native.batch_lock_rows(b._h)[0] == 2
    vals = torch.tensor(values, device="cuda:0")
    g = b.capture("expectation", vals)
    try:
        got = g.replay().clone()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(got.cpu().numpy(), b.expectation(vals).cpu().numpy())
    finally:
        g.close()
    # a call captured while status 2 is injected writes status 1 on the
    # device after its tensor-core launches: every replay marks the
    # tensor-core rows' results (NaN), the queue row's stay exact
    ref = b.expectation(vals).cpu().numpy()
    prev = _native.tc_inject_status(2)
    try:
        g = b.capture("expectation", vals)
    finally:
        _native.tc_inject_status(prev)
    try:
        got = g.replay().clone()
        torch.cuda.synchronize()
        got = got.cpu().numpy()
    finally:
        g.close()
    assert np.isnan(got[[0, 2]]).all()
    np.testing.assert_array_equal(got[1], ref[1])


def test_wide_and_lockstep_rows_in_one_call(lock_tc):
    """A 24-qubit wide row on tensor-core blocks (one launch per block), two
    16-qubit lockstep rows on tensor-core blocks and a resident row in the
    queue, in one expectation call: each path clears and checks the status
    word, and every row matches complex128."""
    from oracle import fast128 as F
    from quantum_gb300 import workloads
    g = workloads.grid_fsim(4, 6, 12, seed=3)
    small, _, sp = _batch([16, 9, 16], [4, 4, 4], 16)
    programs = [g["programs"][0]] + small
    psums = [g["pauli_sums"][0] * 2] + sp
    values = np.zeros((4, len(NAMES)), np.float32)
    values[1:] = np.random.default_rng(5).uniform(-2, 2, size=(3, len(NAMES)))
    prev = _native.set_tensor_core_gates(2)
    try:
        b = ops.Batch(programs, NAMES, psums)
        assert _native.batch_lock_rows(b._h)[0] == 2
        got = b.expectation(values)
        assert _native.tc_blocks(b._h, 0) > 0 and _native.tc_status(b._h) == 0
        assert _native.batch_lock_tc(b._h)[0] > 0
    finally:
        _native.set_tensor_core_gates(prev)
    want = np.zeros_like(got, dtype=np.float64)
    want[0] = F.simulate_expectation_row(programs[0], [], np.zeros(0, np.float32), psums[0])
    want[1:] = O.simulate_expectation(programs[1:], NAMES, values[1:], psums[1:])
    np.testing.assert_allclose(got, want, atol=expectation_atol(psums), rtol=0)
