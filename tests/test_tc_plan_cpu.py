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


def _tf32_rna(x):
    """fp32 -> nearest tf32 (10 mantissa bits), ties away from zero."""
    u = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x1000) & 0xFFFFE000
    return u.astype(np.uint32).view(np.float32)


def _tf32_trunc(x):
    """What the tensor core reads of an fp32 operand: the low 13 bits dropped."""
    return (x.astype(np.float32).view(np.uint32) & np.uint32(0xFFFFE000)).view(np.float32)


def test_split_tf32_arithmetic_of_the_block_kernel():
    """The block kernel's numerics, restated with numpy: the 32 x 32 complex
    block in real form (R[2i][2j] = Re U, R[2i][2j+1] = -Im U, R[2i+1][2j] =
    Im U, R[2i+1][2j+1] = Re U), operands split as hi = rna(x), lo = x - hi,
    D = A_lo R_hi + A_hi R_lo + A_hi R_hi in fp32.  Its error on unit-norm
    states stays below the 1e-6 that the GPU test demands, and a plain TF32
    product misses it by two orders of magnitude."""
    rng = np.random.default_rng(1)
    z = rng.normal(size=(32, 32)) + 1j * rng.normal(size=(32, 32))
    U = np.linalg.qr(z)[0].astype(np.complex64)
    R = np.zeros((64, 64), np.float32)
    R[0::2, 0::2], R[0::2, 1::2] = U.real, -U.imag
    R[1::2, 0::2], R[1::2, 1::2] = U.imag, U.real
    psi = rng.normal(size=(1 << 12)) + 1j * rng.normal(size=(1 << 12))
    psi = (psi / np.linalg.norm(psi)).astype(np.complex64).reshape(128, 32)
    A = np.stack([psi.real, psi.imag], axis=-1).reshape(128, 64).astype(np.float32)
    a_hi, r_hi = _tf32_rna(A), _tf32_rna(R)
    a_lo, r_lo = _tf32_trunc(A - a_hi), _tf32_trunc(R - r_hi)
    f32 = lambda x, y: (x.astype(np.float64) @ y.T.astype(np.float64)).astype(np.float32)
    D = f32(a_lo, r_hi) + f32(a_hi, r_lo) + f32(a_hi, r_hi)
    want = psi.astype(np.complex128) @ U.astype(np.complex128).T
    got = D[:, 0::2] + 1j * D[:, 1::2]
    assert np.abs(got - want).max() < 1e-6
    plain = f32(_tf32_trunc(A), _tf32_trunc(R))
    assert np.abs(plain[:, 0::2] + 1j * plain[:, 1::2] - want).max() > 1e-5
