"""The autotuner on the GPU: for every qubit count of an uneven batch it
times the candidate plans (fusion width 1 or 2; for 15-21 qubits also the
queue or lockstep schedule, and lockstep on 5-qubit tensor-core blocks),
installs the fastest, and batches created afterwards still give the
oracle's expectations."""

import numpy as np
import pytest

from oracle import tfq_oracle as O
from quantum_gb300 import _native, autotune, ops
from quantum_gb300 import serialize as S
from tests.circuits import expectation_atol, random_circuit, random_paulisum

pytestmark = pytest.mark.gpu


def test_tune_installs_the_fastest_candidate(tmp_path, monkeypatch):
    monkeypatch.setenv("TFQG_CACHE_DIR", str(tmp_path))
    rng = np.random.default_rng(5)
    nqs = [5, 5, 11, 11, 17, 17, 17, 14]
    progs, psums = [], []
    for n in nqs:
        qs = S.GridQubit.rect(1, n)
        progs.append(S.serialize_circuit(random_circuit(qs, 5, rng, [])))
        psums.append([random_paulisum(qs, rng)])
    old = _native.set_wide_few_rows(0)
    try:
        res = autotune.tune(progs, psums, samples=100, use_cache=True)
        assert sorted(res) == sorted(set(nqs))
        for n, r in res.items():
            assert r["ms"] == min(r["candidates"].values())
            assert len(r["candidates"]) == (5 if n in autotune.LOCK_QUBITS else 2)
        # a second call installs the cached choices without timing
        again = autotune.tune(progs, psums, samples=100, use_cache=True)
        assert all(r["cached"] for r in again.values())
        b = ops.Batch(progs, [], psums)
        got = b.expectation(np.zeros((len(nqs), 0), np.float32))
        want = O.simulate_expectation(progs, [], np.zeros((len(nqs), 0)), psums)
        np.testing.assert_allclose(got, want, atol=expectation_atol(psums), rtol=0)
    finally:
        autotune.reset()
        _native.set_wide_few_rows(old)
