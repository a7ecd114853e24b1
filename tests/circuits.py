"""Seeded random circuits / Pauli sums for parity tests (test infrastructure).

Shapes follow the reference's fixtures: random moments of the supported gate
set with symbolic exponents (optionally scaled), random controls on some
gates (tensorflow_quantum/python/util.py:94-172), random Pauli sums
(util.py:244-259)."""

import numpy as np

from quantum_gb300 import serialize as S

ONE_Q = ["I", "HP", "XP", "YP", "ZP", "PXP"]
TWO_Q = ["XXP", "YYP", "ZZP", "CZP", "CNP", "SP", "ISP", "FSIM", "PISP"]
CHANNELS = ["DP", "ADP", "GAD", "AD", "RST", "PD", "PF", "BF"]


def _param(rng, symbols, p_sym):
    if symbols and rng.random() < p_sym:
        s = S.Symbol(symbols[rng.integers(len(symbols))])
        return s * float(np.round(rng.uniform(0.2, 1.5), 3)) if rng.random() < 0.5 else s
    return float(rng.uniform(-1.5, 1.5))


def make_gate(rng, gid, qs, symbols, p_sym):
    gs = float(rng.choice([0.0, -0.5, 0.25]))
    if gid == "I":
        return S.I(qs[0])
    if gid == "PXP":
        return S.PhasedXPow(qs[0], _param(rng, symbols, p_sym),
                            _param(rng, symbols, p_sym), gs)
    if gid == "FSIM":
        return S.FSim(qs[0], qs[1], _param(rng, symbols, p_sym),
                      _param(rng, symbols, p_sym))
    if gid == "PISP":
        return S.PhasedISwapPow(qs[0], qs[1], _param(rng, symbols, p_sym),
                                _param(rng, symbols, p_sym))
    ctor = {"HP": S.HPow, "XP": S.XPow, "YP": S.YPow, "ZP": S.ZPow,
            "XXP": S.XXPow, "YYP": S.YYPow, "ZZP": S.ZZPow, "CZP": S.CZPow,
            "CNP": S.CNotPow, "SP": S.SwapPow, "ISP": S.ISwapPow}[gid]
    return ctor(*qs, _param(rng, symbols, p_sym), gs)


def make_channel(rng, cid, q):
    p = float(rng.uniform(0.01, 0.2))
    if cid == "DP":
        return S.depolarize(q, p)
    if cid == "ADP":
        return S.asymmetric_depolarize(q, p / 3, p / 4, p / 5)
    if cid == "GAD":
        return S.generalized_amplitude_damp(q, float(rng.uniform(0, 1)), p)
    if cid == "AD":
        return S.amplitude_damp(q, p)
    if cid == "RST":
        return S.reset(q)
    if cid == "PD":
        return S.phase_damp(q, p)
    if cid == "PF":
        return S.phase_flip(q, p)
    return S.bit_flip(q, p)


def random_circuit(qubits, n_moments, rng, symbols=(), p_sym=0.7,
                   p_control=0.3, density=0.9, channels=(), p_channel=0.0):
    """A circuit on `qubits`; every qubit is touched at least once."""
    qubits = list(qubits)
    moments = []
    for _ in range(n_moments):
        free = list(qubits)
        rng.shuffle(free)
        ops = []
        while free:
            if rng.random() > density:
                free.pop()
                continue
            if channels and rng.random() < p_channel:
                ops.append(make_channel(rng, channels[rng.integers(len(channels))],
                                        free.pop()))
                continue
            two = len(free) >= 2 and rng.random() < 0.5
            gid = (TWO_Q if two else ONE_Q)[rng.integers(len(TWO_Q if two else ONE_Q))]
            k = 2 if two else 1
            qs = [free.pop() for _ in range(k)]
            op = make_gate(rng, gid, qs, list(symbols), p_sym)
            if free and rng.random() < p_control:
                nc = int(rng.integers(1, min(2, len(free)) + 1))
                cs = [free.pop() for _ in range(nc)]
                op = op.controlled_by(*cs, control_values=list(rng.integers(0, 2, nc)))
            ops.append(op)
        moments.append(ops)
    # touch every qubit so the resolved qubit count is len(qubits)
    moments.append([S.I(q) for q in qubits])
    return S.Circuit(moments)


def random_paulisum(qubits, rng, n_terms=4, identity=True):
    qubits = list(qubits)
    terms = []
    for _ in range(n_terms):
        k = int(rng.integers(1, min(4, len(qubits)) + 1))
        sel = rng.choice(len(qubits), size=k, replace=False)
        terms.append((float(rng.normal()),
                      [(qubits[i], "XYZ"[rng.integers(3)]) for i in sel]))
    if identity:
        terms.append((float(rng.normal()), []))
    return S.serialize_paulisum(terms)


def expectation_atol(pauli_sums, per_unit=1e-5):
    """Absolute tolerance for expectations of these Pauli sums: 1e-5 per unit
    of sum_t |c_t| (an error of 1e-5 on each term's <P_t> in [-1, 1]), the
    largest over the batch; identity terms count, as they add exactly."""
    from oracle import tfq_oracle as O
    worst = 1.0
    for row in pauli_sums:
        for ps in row:
            worst = max(worst, sum(abs(float(t["re"])) for t in O.decode_paulisum(ps)))
    return per_unit * worst


def gradient_atol(pauli_sums, downstream_grads, per_unit=1e-5):
    """Absolute tolerance for adjoint gradients: 1e-5 per unit of the
    weighted observable's sum_j |g_j| sum_t |c_t| (lambda's scale), the
    largest over the batch."""
    from oracle import tfq_oracle as O
    g = np.abs(np.asarray(downstream_grads, np.float64))
    worst = 1.0
    for i, row in enumerate(pauli_sums):
        w = sum(g[i, j] * sum(abs(float(t["re"])) for t in O.decode_paulisum(ps))
                for j, ps in enumerate(row))
        worst = max(worst, w)
    return per_unit * worst
