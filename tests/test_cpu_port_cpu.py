"""The timed CPU baseline (oracle/cpu_ref.cc: the reference's expectation and
adjoint loops with a fused forward pass and fused partial blocks) gives the
oracle's answers: random circuits with every gate id and controls, and the
adjoint benchmark's circuit shape at reduced width.  A baseline that
computed something else would time the wrong work."""

import numpy as np
import pytest

from oracle import cpu_port
from oracle import tfq_oracle as O
from quantum_gb300 import serialize as S
from quantum_gb300 import workloads
from tests.circuits import random_circuit, random_paulisum


@pytest.mark.parametrize("nqs,seed", [([1, 3, 5], 0), ([6, 8], 1), ([4, 7], 2)])
def test_random_circuits_match_oracle(nqs, seed):
    rng = np.random.default_rng(seed)
    names = [f"s{i}" for i in range(5)]
    progs, psums = [], []
    for n in nqs:
        qs = S.GridQubit.rect(1, n)
        progs.append(S.serialize_circuit(random_circuit(qs, 6, rng, names, p_control=0.3)))
        psums.append([random_paulisum(qs, rng) for _ in range(2)])
    vals = rng.uniform(-2, 2, size=(len(nqs), 5)).astype(np.float32)
    dg = rng.normal(size=(len(nqs), 2)).astype(np.float32)
    flat = cpu_port.Flat(progs, names, vals, psums)
    e, g = flat.run(dg, threads=2)
    we = O.simulate_expectation(progs, names, vals, psums)
    wg = O.adj_grad(progs, names, vals, psums, dg)
    np.testing.assert_allclose(e, we, atol=2e-5 * max(1, np.abs(we).max()), rtol=0)
    np.testing.assert_allclose(g, wg, atol=2e-5 * max(1, np.abs(wg).max()), rtol=0)


def test_hea_shape_matches_oracle():
    w = workloads.adjoint_hea(batch=3, n=8, depth=4, seed=5)
    flat = cpu_port.Flat(w["programs"], w["symbol_names"], w["symbol_values"],
                         w["pauli_sums"])
    e, g = flat.run(w["downstream_grads"], threads=3)
    we = O.simulate_expectation(w["programs"], w["symbol_names"], w["symbol_values"],
                                w["pauli_sums"])
    wg = O.adj_grad(w["programs"], w["symbol_names"], w["symbol_values"],
                    w["pauli_sums"], w["downstream_grads"])
    np.testing.assert_allclose(e, we, atol=1e-5, rtol=0)
    np.testing.assert_allclose(g, wg, atol=2e-5 * max(1, np.abs(wg).max()), rtol=0)
    e2, g2 = flat.run(w["downstream_grads"], threads=1, adjoint=False)
    np.testing.assert_allclose(e2, e, atol=0, rtol=0)
    assert not g2.any()
