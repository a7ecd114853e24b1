"""Seeded synthetic workloads with the benchmark configurations' shapes.

The reference publishes no benchmark data and names no dataset; these
generators build the circuits, symbol values and observables the benchmark
configurations describe, encoded exactly as the reference serializer would.
"""

import math

import numpy as np

from . import serialize as S


def tfim(qubits, rng):
    """sum_i J_i Z_i Z_{i+1} + sum_i h_i X_i with J, h ~ N(1, 0.1)."""
    n = len(qubits)
    J = rng.normal(1.0, 0.1, size=n - 1)
    h = rng.normal(1.0, 0.1, size=n)
    terms = [(float(J[i]), [(qubits[i], "Z"), (qubits[i + 1], "Z")])
             for i in range(n - 1)]
    terms += [(float(h[i]), [(qubits[i], "X")]) for i in range(n)]
    return S.serialize_paulisum(terms)


def adjoint_hea(batch=256, n=16, depth=10, seed=1):
    """Hardware-efficient ansatz for the adjoint-gradient benchmark: per layer
    Ry and Rz (symbolic) on every qubit, then a CNOT ladder 0->1->...->n-1;
    symbol values U[0, 2pi); one TFIM observable; downstream grads = 1."""
    rng = np.random.default_rng(seed)
    qs = S.GridQubit.rect(1, n)
    names = []
    moments = []
    for layer in range(depth):
        ys = [f"ry_{layer}_{i}" for i in range(n)]
        zs = [f"rz_{layer}_{i}" for i in range(n)]
        names += ys + zs
        moments.append([S.ry(qs[i], S.Symbol(ys[i])) for i in range(n)])
        moments.append([S.rz(qs[i], S.Symbol(zs[i])) for i in range(n)])
        for i in range(n - 1):
            moments.append([S.CNOT(qs[i], qs[i + 1])])
    prog = S.serialize_circuit(S.Circuit(moments))
    values = rng.uniform(0, 2 * math.pi, size=(batch, len(names))).astype(np.float32)
    ps = tfim(qs, rng)
    return dict(programs=[prog] * batch, symbol_names=names, symbol_values=values,
                pauli_sums=[[ps] for _ in range(batch)],
                downstream_grads=np.ones((batch, 1), np.float32),
                n=n, depth=depth, num_gates=depth * (2 * n + n - 1))


def expectation_layers(batch=32, n=12, layers=20, seed=1):
    """Rx, Ry, Rz (symbolic) on every qubit per layer, then a brick-wall of CZ
    (even pairs on even layers, odd pairs on odd layers); 4 observables:
    sum Z_i, sum Z_i Z_{i+1}, sum X_i, 10 random Pauli strings with N(0,1)
    coefficients."""
    rng = np.random.default_rng(seed)
    qs = S.GridQubit.rect(1, n)
    names, moments = [], []
    for layer in range(layers):
        for axis, ctor in (("x", S.rx), ("y", S.ry), ("z", S.rz)):
            syms = [f"r{axis}_{layer}_{i}" for i in range(n)]
            names += syms
            moments.append([ctor(qs[i], S.Symbol(syms[i])) for i in range(n)])
        start = layer % 2
        moments.append([S.CZ(qs[i], qs[i + 1]) for i in range(start, n - 1, 2)])
    prog = S.serialize_circuit(S.Circuit(moments))
    values = rng.uniform(0, 2 * math.pi, size=(batch, len(names))).astype(np.float32)
    rand_terms = []
    for _ in range(10):
        paulis = [(qs[i], "XYZ"[rng.integers(3)]) for i in range(n)
                  if rng.random() < 0.5]
        rand_terms.append((float(rng.normal()), paulis))
    ops = [S.serialize_paulisum([(1.0, [(q, "Z")]) for q in qs]),
           S.serialize_paulisum([(1.0, [(qs[i], "Z"), (qs[i + 1], "Z")])
                                 for i in range(n - 1)]),
           S.serialize_paulisum([(1.0, [(q, "X")]) for q in qs]),
           S.serialize_paulisum(rand_terms)]
    n_cz = sum(len(range(layer % 2, n - 1, 2)) for layer in range(layers))
    n_terms = n + (n - 1) + n + len(rand_terms)
    return dict(programs=[prog] * batch, symbol_names=names, symbol_values=values,
                pauli_sums=[list(ops) for _ in range(batch)], n=n,
                counts=dict(one=3 * n * layers, two=n_cz, channels=0, terms=n_terms))


def uneven_batch(batch=4096, n_min=4, n_max=20, d_min=5, d_max=40, seed=1):
    """Random circuits with n ~ U{n_min..n_max} qubits and U{d_min..d_max}
    layers; a layer is a random-axis rotation (angle U[0, 2pi)) on every
    qubit, then random disjoint pairs with CZ or ISWAP^t (t ~ U[0, 1]).
    Observable sum_i Z_i."""
    rng = np.random.default_rng(seed)
    programs, psums, ns = [], [], []
    for _ in range(batch):
        n = int(rng.integers(n_min, n_max + 1))
        ns.append(n)
        depth = int(rng.integers(d_min, d_max + 1))
        qs = S.GridQubit.rect(1, n)
        moments = []
        for _ in range(depth):
            rot = []
            for q in qs:
                axis = int(rng.integers(3))
                theta = float(rng.uniform(0, 2 * math.pi))
                rot.append((S.rx, S.ry, S.rz)[axis](q, theta))
            moments.append(rot)
            perm = rng.permutation(n)
            pairs = []
            for k in range(0, n - 1, 2):
                a, b = qs[perm[k]], qs[perm[k + 1]]
                if rng.random() < 0.5:
                    pairs.append(S.CZ(a, b))
                else:
                    pairs.append(S.ISwapPow(a, b, float(rng.uniform(0, 1))))
            moments.append(pairs)
        programs.append(S.serialize_circuit(S.Circuit(moments)))
        psums.append([S.serialize_paulisum([(1.0, [(q, "Z")]) for q in qs])])
    return dict(programs=programs, symbol_names=[],
                symbol_values=np.zeros((batch, 0), np.float32), pauli_sums=psums,
                n_per_row=ns)


def noisy_brickwall(batch=64, n=14, depth=15, p=0.01, seed=1):
    """Ry, Rz (angles U[0, 2pi)) + CZ brick-wall per layer, a depolarizing
    channel DP(p) after every gate on each qubit it touched; observable
    sum_i Z_i."""
    rng = np.random.default_rng(seed)
    qs = S.GridQubit.rect(1, n)
    programs = []
    for _ in range(batch):
        moments = []
        for layer in range(depth):
            for ctor in (S.ry, S.rz):
                moments.append([ctor(q, float(rng.uniform(0, 2 * math.pi))) for q in qs])
                moments.append([S.depolarize(q, p) for q in qs])
            start = layer % 2
            cz = [(qs[i], qs[i + 1]) for i in range(start, n - 1, 2)]
            moments.append([S.CZ(a, b) for a, b in cz])
            moments.append([S.depolarize(q, p) for a, b in cz for q in (a, b)])
        programs.append(S.serialize_circuit(S.Circuit(moments)))
    ps = S.serialize_paulisum([(1.0, [(q, "Z")]) for q in qs])
    n_cz = sum(len(range(layer % 2, n - 1, 2)) for layer in range(depth))
    return dict(programs=programs, symbol_names=[],
                symbol_values=np.zeros((batch, 0), np.float32),
                pauli_sums=[[ps] for _ in range(batch)], n=n, p=p,
                counts=dict(one=2 * n * depth, two=n_cz,
                            channels=2 * n * depth + 2 * n_cz, terms=n))


def grid_fsim(rows=5, cols=6, depth=24, seed=1):
    """One random circuit on a rows x cols GridQubit array (30 qubits at the
    default size). Each layer applies one of {sqrt(X), sqrt(Y), sqrt(W)} to
    every qubit, never the gate that qubit had in the previous layer, where
    sqrt(W) = PhasedXPow(0.25, 0.5). Then fSim(theta ~ U[1.4, 1.7],
    phi ~ U[0.4, 0.6]) runs on one of four coupler patterns, cycled:
    horizontal pairs at even / odd columns, then vertical pairs at even /
    odd rows. Observable sum_i Z_i."""
    rng = np.random.default_rng(seed)
    qs = [S.GridQubit(r, c) for r in range(rows) for c in range(cols)]
    at = {(q.row, q.col): q for q in qs}
    last = [-1] * len(qs)
    moments = []
    for layer in range(depth):
        one = []
        for i, q in enumerate(qs):
            g = int(rng.integers(3))
            if g == last[i]:
                g = (g + 1 + int(rng.integers(2))) % 3
            last[i] = g
            one.append(S.XPow(q, 0.5) if g == 0 else S.YPow(q, 0.5) if g == 1
                       else S.PhasedXPow(q, 0.25, 0.5))
        moments.append(one)
        pattern = layer % 4
        pairs = []
        for r in range(rows):
            for c in range(cols):
                if pattern < 2 and c % 2 == pattern and c + 1 < cols:
                    pairs.append((at[r, c], at[r, c + 1]))
                if pattern >= 2 and r % 2 == pattern - 2 and r + 1 < rows:
                    pairs.append((at[r, c], at[r + 1, c]))
        moments.append([S.FSim(a, b, float(rng.uniform(1.4, 1.7)),
                               float(rng.uniform(0.4, 0.6))) for a, b in pairs])
    prog = S.serialize_circuit(S.Circuit(moments))
    ps = S.serialize_paulisum([(1.0, [(q, "Z")]) for q in qs])
    n_two = sum(len(m) for m in moments[1::2])
    return dict(programs=[prog], symbol_names=[],
                symbol_values=np.zeros((1, 0), np.float32), pauli_sums=[[ps]],
                n=len(qs), depth=depth,
                counts=dict(one=len(qs) * depth, two=n_two, channels=0, terms=len(qs)))
