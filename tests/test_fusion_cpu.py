"""Gate fusion of forward plans, checked on the host (no GPU).

The gates of a row's forward plan, with matrices bound on the host by the
same product code the device runs for a fused gate (gate_math.cuh), are
applied with numpy in plan order and compared with the oracle's state of the
unfused circuit. Fused plans must also hold fewer gates where the cost model
says fusion pays (one-qubit chains beside dense two-qubit gates)."""

import numpy as np
import pytest

from oracle import tfq_oracle as O
from quantum_gb300 import _native, ops, workloads
from quantum_gb300 import serialize as S
from tests.circuits import random_circuit

GK_FUSED = 32


def _apply(psi, n, m, nq, b0, b1, cmask, cval):
    idx = np.arange(1 << n)
    sel = (idx & cmask) == cval
    if nq == 1:
        x0 = idx[sel & (((idx >> b0) & 1) == 0)]
        x1 = x0 | (1 << b0)
        a0, a1 = psi[x0].copy(), psi[x1].copy()
        psi[x0] = m[0, 0] * a0 + m[0, 1] * a1
        psi[x1] = m[1, 0] * a0 + m[1, 1] * a1
        return
    base = idx[sel & (((idx >> b0) & 1) == 0) & (((idx >> b1) & 1) == 0)]
    xs = [base | (r0 << b0) | (r1 << b1) for r0 in (0, 1) for r1 in (0, 1)]
    a = [psi[x].copy() for x in xs]
    for r in range(4):
        psi[xs[r]] = sum(m[r, c] * a[c] for c in range(4))


def _plan_states(programs, names, values, ns, fuse):
    prev = _native.set_gate_fusion(fuse)
    try:
        b = ops.Batch(programs, names, None, kind=ops.KIND_FORWARD)
    finally:
        _native.set_gate_fusion(prev)
    states, counts = [], []
    for row in range(len(programs)):
        gates = _native.forward_plan_gates(b._h, row, values[row])
        n = ns[row]
        psi = np.zeros(1 << n, np.complex128)
        psi[0] = 1.0
        for nq, b0, b1, cmask, cval, _, m in gates:
            _apply(psi, n, m, nq, b0, b1, cmask, cval)
        states.append(psi)
        counts.append((len(gates), sum(g[5] == GK_FUSED for g in gates)))
    b.close()
    return states, counts


def _check(programs, names, values, tol=2e-6):
    ref = O.simulate_state(programs, names, values)
    ns = [p[0] for p in O._parse_all(programs, names, values)[0]]
    out = {}
    for fuse in (False, True):
        states, counts = _plan_states(programs, names, values, ns, fuse)
        for i, psi in enumerate(states):
            np.testing.assert_allclose(psi, ref[i, : psi.size], atol=tol, rtol=0)
        out[fuse] = counts
    return out


def test_random_circuits_fused_plan_matches_oracle():
    rng = np.random.default_rng(5)
    names = ["a", "b", "c"]
    programs, rows = [], []
    for n in (2, 3, 5, 7, 9):
        qs = S.GridQubit.rect(1, n)
        for _ in range(3):
            c = random_circuit(qs, 12, rng, names, p_control=0.25)
            programs.append(S.serialize_circuit(c))
    values = rng.uniform(-2, 2, size=(len(programs), len(names))).astype(np.float32)
    counts = _check(programs, names, values)
    assert any(f for _, f in counts[True]), "no gate was fused"


def test_rotation_chains_and_cz_brickwall():
    w = workloads.expectation_layers(batch=3, n=6, layers=4, seed=3)
    counts = _check(w["programs"], w["symbol_names"], w["symbol_values"])
    # Rx Ry Rz chains merge and fold into the CZs: far fewer gates
    assert counts[True][0][0] * 2 < counts[False][0][0]


def test_grid_fsim_absorbs_single_qubit_gates():
    w = workloads.grid_fsim(rows=3, cols=3, depth=8, seed=2)
    values = np.zeros((1, 0), np.float32)
    counts = _check(w["programs"], [], values)
    total_fused, fused = counts[True][0]
    # every one-qubit gate lands in an fSim: only the fSims remain
    n_fsim = w["programs"][0].count(b"FSIM") if isinstance(w["programs"][0], bytes) else None
    assert fused > 0 and total_fused * 2 < counts[False][0][0]
    if n_fsim:
        assert total_fused == n_fsim


def test_uneven_batch_rows():
    w = workloads.uneven_batch(batch=6, n_min=3, n_max=8, d_min=3, d_max=8, seed=4)
    _check(w["programs"], [], w["symbol_values"])


def test_controls_block_fusion():
    """A controlled gate on a chain's qubit ends the chain: the one-qubit
    gates on either side of it must not meet in one fused gate."""
    q = S.GridQubit.rect(1, 3)
    c = S.Circuit([[S.rx(q[0], 0.3)], [S.ry(q[0], 0.7)],
                   [S.XPow(q[0], 0.4).controlled_by(q[1])],
                   [S.rz(q[0], 1.1)], [S.HPow(q[0], 0.6)],
                   [S.FSim(q[0], q[2], 1.5, 0.5)], [S.rx(q[2], 0.2)],
                   [S.CZ(q[1], q[2])], [S.ry(q[1], 0.9)]])
    programs = [S.serialize_circuit(c)]
    _check(programs, [], np.zeros((1, 0), np.float32))


@pytest.mark.parametrize("n", [1, 2])
def test_tiny_programs(n):
    q = S.GridQubit.rect(1, n)
    moments = [[S.rx(q[0], 0.3)], [S.rz(q[0], 0.2)], [S.ry(q[0], 0.1)]]
    if n == 2:
        moments += [[S.CZ(q[0], q[1])], [S.rx(q[1], 0.5)]]
    _check([S.serialize_circuit(S.Circuit(moments))], [], np.zeros((1, 0), np.float32))
