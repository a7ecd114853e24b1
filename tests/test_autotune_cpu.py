"""The per-qubit-count row policy that the autotuner installs
(tfqg_internal_set_row_policy) reaches the host plans of batches created
afterwards, without a GPU: gate fusion per qubit count (the forward plan of a
row has fewer, fused gates when it is on) and lockstep rows per qubit count;
and the autotuner's qubit counts are the resolved ones."""

import numpy as np

from quantum_gb300 import _native, autotune, ops
from quantum_gb300 import serialize as S
from tests.circuits import random_circuit


def _batch(nqs, seed=0):
    rng = np.random.default_rng(seed)
    progs = [S.serialize_circuit(random_circuit(S.GridQubit.rect(1, n), 6, rng, []))
             for n in nqs]
    return progs


def test_fusion_and_lockstep_follow_the_row_policy():
    progs = _batch([12, 18, 18, 6, 18])
    old = _native.set_wide_few_rows(0)
    try:
        autotune.reset()
        b = ops.Batch(progs, [], None)
        fused = len(_native.forward_plan_gates(b._h, 0, np.zeros(0, np.float32)))
        assert _native.batch_lock_rows(b._h)[0] == 3
        autotune.set_row_policy(12, fuse=0)
        autotune.set_row_policy(18, lock=0)
        b2 = ops.Batch(progs, [], None)
        unfused = len(_native.forward_plan_gates(b2._h, 0, np.zeros(0, np.float32)))
        assert unfused > fused
        assert _native.batch_lock_rows(b2._h)[0] == 0
        autotune.reset()
        b3 = ops.Batch(progs, [], None)
        assert len(_native.forward_plan_gates(b3._h, 0, np.zeros(0, np.float32))) == fused
        assert _native.batch_lock_rows(b3._h)[0] == 3
    finally:
        autotune.reset()
        _native.set_wide_few_rows(old)


def test_qubit_counts_are_resolved_counts():
    assert autotune.qubit_counts(_batch([3, 9, 1])) == [3, 9, 1]
