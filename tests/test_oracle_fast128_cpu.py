"""The oracle's compiled complex128 loops (oracle/sv128.c via
oracle/fast128.py) against the numpy oracle on small circuits: states with
controlled gates of every id, density matrices with all eight channels, and
Pauli-string traces.  These loops back the large-size checks (24-qubit
states, 14-qubit density matrices), so they are pinned here first."""

import numpy as np
import pytest

from oracle import fast128 as F
from oracle import tfq_oracle as O
from quantum_gb300 import serialize as S
from tests.circuits import CHANNELS, random_circuit, random_paulisum


@pytest.mark.parametrize("n,seed", [(1, 0), (4, 1), (7, 2)])
def test_state_matches_numpy_oracle(n, seed):
    rng = np.random.default_rng(seed)
    qs = S.GridQubit.rect(1, n)
    names = ["a", "b", "c"]
    prog = S.serialize_circuit(random_circuit(qs, 6, rng, names, p_control=0.4))
    vals = rng.uniform(-2, 2, size=3).astype(np.float32)
    want = O.simulate_state([prog], names, vals[None, :])[0]
    nn, _, got = F.simulate_state_row(prog, names, vals)
    assert nn == n
    np.testing.assert_allclose(got, want[:2 ** n], atol=1e-12, rtol=0)
    ps = [random_paulisum(qs, rng) for _ in range(3)]
    want_e = O.simulate_expectation([prog], names, vals[None, :], [ps])[0]
    got_e = F.simulate_expectation_row(prog, names, vals, ps)
    np.testing.assert_allclose(got_e, want_e, atol=1e-12, rtol=0)


@pytest.mark.parametrize("n,seed", [(2, 3), (4, 4)])
def test_density_matrix_matches_numpy_oracle(n, seed):
    rng = np.random.default_rng(seed)
    qs = S.GridQubit.rect(1, n)
    names = ["a"]
    progs, psums = [], []
    for _ in range(2):
        c = random_circuit(qs, 6, rng, names, p_control=0.3, channels=CHANNELS,
                           p_channel=0.4)
        progs.append(S.serialize_circuit(c))
        psums.append([random_paulisum(qs, rng), random_paulisum(qs, rng)])
    vals = rng.uniform(-1, 1, size=(2, 1)).astype(np.float32)
    parsed, _ = O._parse_all(progs, names, vals, None, noisy=True)
    for nn, _, items in parsed:
        want = O._final_dm(nn, items).reshape(-1)
        got = F.final_dm(nn, items)
        np.testing.assert_allclose(got, want, atol=1e-12, rtol=0)
    want_e = O.noisy_expectation_exact(progs, names, vals, psums)
    got_e = F.noisy_expectation_exact(progs, names, vals, psums)
    np.testing.assert_allclose(got_e, want_e, atol=1e-12, rtol=0)
