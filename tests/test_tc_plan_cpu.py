"""Tensor-core block plans of wide rows, checked on the host (no GPU).

plan_tc_blocks groups a forward program's gates into blocks of at most 5
qubits; each block's 32 x 32 matrix is the product of its members, built by
the same code the device runs (gate_math.cuh tc_block_column).  Applying the
blocks in order with numpy must give the oracle's state of the circuit, which
pins the planner's reordering (a gate only moves past blocks it commutes
with), the padding bits and the block matrices.  Rows need at least 12
qubits (one chunk of 128 groups of 32 amplitudes)."""

import numpy as np
import pytest

from oracle import tfq_oracle as O
from quantum_gb300 import _native, ops, workloads
from quantum_gb300 import serialize as S
from tests.circuits import random_circuit


def _apply_block(psi, n, tgt, U):
    idx = np.arange(1 << n)
    tmask = sum(1 << t for t in tgt)
    base = idx[(idx & tmask) == 0]
    off = np.array([sum(((j >> i) & 1) << t for i, t in enumerate(tgt))
                    for j in range(32)])
    pos = base[:, None] + off[None, :]
    psi[pos] = psi[pos] @ U.T


def _check(programs, names, values, tol=2e-6):
    b = ops.Batch(programs, names, None, kind=ops.KIND_FORWARD)
    ref = O.simulate_state(programs, names, values)
    ns = [p[0] for p in O._parse_all(programs, names, values)[0]]
    counts = []
    for row, n in enumerate(ns):
        plan = _native.tc_plan(b._h, row, values[row])
        assert plan is not None
        psi = np.zeros(1 << n, np.complex128)
        psi[0] = 1.0
        for tgt, U in plan:
            assert list(tgt) == sorted(set(tgt)) and len(tgt) == 5 and max(tgt) < n
            np.testing.assert_allclose(U @ U.conj().T, np.eye(32), atol=1e-6)
            _apply_block(psi, n, tgt, U)
        np.testing.assert_allclose(psi, ref[row, : psi.size], atol=tol, rtol=0)
        counts.append(len(plan))
    b.close()
    return counts


def test_random_circuits_with_controls():
    rng = np.random.default_rng(11)
    names = ["a", "b", "c"]
    programs = []
    for n in (12, 13):
        qs = S.GridQubit.rect(1, n)
        for _ in range(2):
            # one control at most: every gate spans at most 3 qubits
            c = random_circuit(qs, 10, rng, names, p_control=0.2)
            programs.append(S.serialize_circuit(c))
    values = rng.uniform(-2, 2, size=(len(programs), len(names))).astype(np.float32)
    _check(programs, names, values)


def test_grid_fsim_blocks_hold_several_gates():
    w = workloads.grid_fsim(rows=3, cols=4, depth=8, seed=3)
    values = np.zeros((1, 0), np.float32)
    nblocks = _check(w["programs"], [], values)[0]
    b = ops.Batch(w["programs"], [], None, kind=ops.KIND_FORWARD)
    ngates = len(_native.forward_plan_gates(b._h, 0, values[0]))
    b.close()
    # the fused forward plan leaves one gate per fSim; blocks hold several
    assert nblocks * 2 < ngates


def test_rotation_layers():
    w = workloads.expectation_layers(batch=2, n=12, layers=3, seed=5)
    _check(w["programs"], w["symbol_names"], w["symbol_values"])


def test_small_rows_have_no_plan():
    q = S.GridQubit.rect(1, 8)
    programs = [S.serialize_circuit(S.Circuit([[S.rx(q[0], 0.3)], [S.CZ(q[0], q[1])]]))]
    b = ops.Batch(programs, [], None, kind=ops.KIND_FORWARD)
    assert _native.tc_plan(b._h, 0, np.zeros(0, np.float32)) is None
    b.close()


def test_gate_on_six_qubits_has_no_plan():
    """A gate with 4 controls and 2 targets spans 6 bits: no 5-bit block
    holds it, so the row keeps the tile passes."""
    q = S.GridQubit.rect(1, 12)
    wide_gate = S.CZ(q[0], q[1]).controlled_by(q[2], q[3], q[4], q[5])
    programs = [S.serialize_circuit(S.Circuit([[S.rx(q[6], 0.3)], [wide_gate]]))]
    b = ops.Batch(programs, [], None, kind=ops.KIND_FORWARD)
    assert _native.tc_plan(b._h, 0, np.zeros(0, np.float32)) is None
    b.close()


def test_deep_random_circuits_with_two_controls():
    """Deeper random circuits on 12 qubits, up to two controls per gate
    (4-qubit gates): the reordering across blocks must keep every
    dependency on targets and controls."""
    rng = np.random.default_rng(23)
    names = ["a", "b"]
    qs = S.GridQubit.rect(1, 12)
    programs = [S.serialize_circuit(random_circuit(qs, 24, rng, names, p_control=0.5))
                for _ in range(2)]
    values = rng.uniform(-2, 2, size=(len(programs), len(names))).astype(np.float32)
    _check(programs, names, values)


def test_noisy_program_has_no_plan():
    """Channels are not gates: a noisy program keeps its tile passes."""
    rng = np.random.default_rng(4)
    qs = S.GridQubit.rect(1, 12)
    c = random_circuit(qs, 4, rng, (), channels=("DP", "AD"), p_channel=0.3)
    b = ops.Batch([S.serialize_circuit(c)], [], None, kind=ops.KIND_NOISY)
    assert _native.tc_plan(b._h, 0, np.zeros(0, np.float32)) is None
    b.close()
