"""Tensor-core forward path of wide rows (tc_gates.cu) on the GPU.

The block kernel alone: a random 5-qubit unitary applied to a random state
on several target sets (the lowest bits, scattered bits, the highest bits;
sets with a target among bits 0-4 take the kernel's transposed variant),
against numpy in complex128.  Split 3xTF32 must keep fp32-level accuracy:
1e-6 absolute on states of unit norm, where a plain-TF32 product is off by
about 4e-5 at 12 qubits (test_tc_plan_cpu.py restates both with numpy).
Then whole wide rows with the tensor-core path switched on: states and
expectations against the oracle at the tolerances of test_gpu_parity.py
(1e-5 states, 8e-5 expectations)."""

import numpy as np
import pytest

from oracle import tfq_oracle as O
from quantum_gb300 import _native, ops, workloads
from quantum_gb300 import serialize as S
from tests.circuits import expectation_atol, random_circuit, random_paulisum

pytestmark = pytest.mark.gpu


def _unitary(rng, d=32):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _apply_np(psi, n, tgt, U):
    idx = np.arange(1 << n)
    tmask = sum(1 << t for t in tgt)
    base = idx[(idx & tmask) == 0]
    off = np.array([sum(((j >> i) & 1) << t for i, t in enumerate(tgt)) for j in range(32)])
    pos = base[:, None] + off[None, :]
    out = psi.copy()
    out[pos] = psi[pos] @ U.T
    return out


@pytest.mark.parametrize("n,tgt,grid", [
    (12, (0, 1, 2, 3, 4), 0),
    (14, (3, 7, 8, 12, 13), 0),
    (14, (9, 10, 11, 12, 13), 1),
    (13, (0, 5, 6, 11, 12), 2),
    (13, (2, 3, 4, 5, 6), 0),
    (14, (4, 10, 11, 12, 13), 0),
    (12, (1, 2, 7, 8, 11), 3),
])
def test_block_kernel_matches_complex128(n, tgt, grid):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(n * 100 + tgt[0])
    U = _unitary(rng).astype(np.complex64)
    psi = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n))
    psi = (psi / np.linalg.norm(psi)).astype(np.complex64)
    tpsi = torch.tensor(psi, device=dev)
    tU = torch.tensor(U, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream().cuda_stream
    want = psi.astype(np.complex128)
    for _ in range(2):  # two launches in a row on the same state
        _native.tc_apply(tpsi.data_ptr(), n, tU.data_ptr(), tgt, st.data_ptr(), s, grid)
        want = _apply_np(want, n, tgt, U.astype(np.complex128))
    torch.cuda.synchronize()
    assert int(st.item()) == 0, "MMA completion wait timed out"
    got = tpsi.cpu().numpy()
    assert np.abs(got - want).max() < 1e-6


@pytest.fixture
def tensor_core_wide():
    old_w = _native.set_wide_min_qubits(15)
    old_t = _native.set_tensor_core_gates(True)
    yield
    _native.set_tensor_core_gates(old_t)
    _native.set_wide_min_qubits(old_w)


def test_wide_rows_state_and_expectation(tensor_core_wide):
    rng = np.random.default_rng(21)
    names = ["a", "b", "c", "d"]
    nqs = [15, 6, 17]
    programs, psums = [], []
    for n in nqs:
        qs = S.GridQubit.rect(1, n)
        programs.append(S.serialize_circuit(random_circuit(qs, 8, rng, names, p_control=0.2)))
        psums.append([random_paulisum(qs, rng, n_terms=6) for _ in range(2)])
    values = rng.uniform(-2, 2, size=(len(nqs), len(names))).astype(np.float32)
    b = ops.Batch(programs, names, psums)
    assert _native.batch_wide_rows(b._h) == 2
    got_e = b.expectation(values)
    assert _native.tc_blocks(b._h, 0) > 0 and _native.tc_blocks(b._h, 1) > 0
    np.testing.assert_allclose(got_e, O.simulate_expectation(programs, names, values, psums),
                               atol=expectation_atol(psums), rtol=0)
    sb = ops.Batch(programs, names, None)
    got_s = sb.state(values)
    np.testing.assert_allclose(got_s, O.simulate_state(programs, names, values),
                               atol=1e-5, rtol=0)
    assert _native.tc_status(b._h) == 0 and _native.tc_status(sb._h) == 0


def test_grid_fsim_row_matches_oracle_and_tile_passes(tensor_core_wide):
    w = workloads.grid_fsim(rows=3, cols=6, depth=10, seed=4)
    values = np.zeros((1, 0), np.float32)
    b = ops.Batch(w["programs"], [], None)
    got = b.state(values)
    assert _native.tc_blocks(b._h, 0) > 0 and _native.tc_status(b._h) == 0
    want = O.simulate_state(w["programs"], [], values)
    np.testing.assert_allclose(got, want, atol=1e-5, rtol=0)
    _native.set_tensor_core_gates(False)
    tile = ops.Batch(w["programs"], [], None).state(values)
    np.testing.assert_allclose(got, tile, atol=1e-5, rtol=0)


def test_auto_mode_takes_rows_of_24_qubits():
    """By default only rows of 24+ qubits (states beyond L2) run the blocks;
    a 24-qubit grid circuit agrees with the tile passes on <sum Z>."""
    old_w = _native.set_wide_min_qubits(15)
    old_t = _native.set_tensor_core_gates("auto")
    try:
        small = workloads.grid_fsim(rows=3, cols=6, depth=4, seed=5)
        b = ops.Batch(small["programs"], [], small["pauli_sums"])
        b.expectation(small["symbol_values"])
        assert _native.tc_blocks(b._h, 0) == -1
        w = workloads.grid_fsim(rows=4, cols=6, depth=8, seed=6)
        b = ops.Batch(w["programs"], [], w["pauli_sums"])
        got = b.expectation(w["symbol_values"])
        assert _native.tc_blocks(b._h, 0) > 0 and _native.tc_status(b._h) == 0
        _native.set_tensor_core_gates(False)
        tile = ops.Batch(w["programs"], [], w["pauli_sums"]).expectation(w["symbol_values"])
        np.testing.assert_allclose(got, tile, atol=1e-5, rtol=0)
    finally:
        _native.set_tensor_core_gates(old_t)
        _native.set_wide_min_qubits(old_w)


def test_block_timeout_fails_the_call_and_is_not_sticky(tensor_core_wide):
    """A block kernel whose MMA wait timed out leaves its row partly
    transformed: the call must fail with INTERNAL instead of returning that
    row, and the next call on the same batch must not inherit the failure.
    The timeout is injected on the host (the status word the host reads
    back), so nothing waits on the GPU."""
    rng = np.random.default_rng(31)
    qs = S.GridQubit.rect(1, 17)
    programs = [S.serialize_circuit(random_circuit(qs, 6, rng, []))]
    psums = [[random_paulisum(qs, rng)]]
    values = np.zeros((1, 0), np.float32)
    b = ops.Batch(programs, [], psums)
    prev = _native.tc_inject_status(1)
    try:
        with pytest.raises(_native.InternalError, match="timed out"):
            b.expectation(values)
        with pytest.raises(_native.InternalError, match="timed out"):
            ops.Batch(programs, [], None).state(values)
    finally:
        _native.tc_inject_status(prev)
    got = b.expectation(values)
    assert _native.tc_blocks(b._h, 0) > 0 and _native.tc_status(b._h) == 0
    np.testing.assert_allclose(got, O.simulate_expectation(programs, [], values, psums),
                               atol=expectation_atol(psums), rtol=0)


def test_two_block_sweeps_match_single_block_sweeps(tensor_core_wide):
    """A wide row whose consecutive blocks share sweeps (tc_sweep_kernel)
    gives the state of one sweep per block, with fewer sweeps."""
    w = workloads.grid_fsim(rows=4, cols=5, depth=12, seed=8)
    values = np.zeros((1, 0), np.float32)
    b = ops.Batch(w["programs"], [], None)
    prev = _native.set_tc_sweep(True)
    try:
        paired = b.state(values)
        blocks, sweeps = _native.tc_blocks(b._h, 0), _native.tc_sweeps(b._h, 0)
        assert blocks > 0 and 0 < sweeps < blocks and _native.tc_status(b._h) == 0
        _native.set_tc_sweep(False)
        single = b.state(values)
        assert _native.tc_sweeps(b._h, 0) == blocks
    finally:
        _native.set_tc_sweep(prev)
    np.testing.assert_allclose(paired, single, atol=1e-6, rtol=0)
    np.testing.assert_allclose(paired, O.simulate_state(w["programs"], [], values),
                               atol=1e-5, rtol=0)
