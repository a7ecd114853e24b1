"""ShardedBatch on one GPU: the shards of every rank of a 3-way split, run
one after another and concatenated, reproduce the whole batch (expectation,
adjoint gradient, padded states, sample layout)."""

import numpy as np
import pytest

from oracle import tfq_oracle as O
from quantum_gb300 import ops, sharding
from tests.circuits import expectation_atol, gradient_atol
from tests.test_sharding_gloo import _uneven

pytestmark = pytest.mark.gpu


def test_three_way_split_reproduces_the_whole_batch():
    programs, names, values, psums = _uneven()
    dg = np.linspace(-1, 1, 2 * len(programs)).reshape(-1, 2).astype(np.float32)
    shards = [sharding.ShardedBatch(programs, names, psums, kind=ops.KIND_ADJOINT,
                                    rank=r, world=3) for r in range(3)]
    exp = np.concatenate([s.expectation(values) for s in shards])
    grad = np.concatenate([s.adj_grad(values, dg) for s in shards])
    np.testing.assert_allclose(exp, O.simulate_expectation(programs, names, values, psums),
                               atol=expectation_atol(psums), rtol=0)
    want = O.adj_grad(programs, names, values, psums, dg)
    np.testing.assert_allclose(grad, want, atol=gradient_atol(psums, dg), rtol=0)
    fwd = [sharding.ShardedBatch(programs, names, None, rank=r, world=3) for r in range(3)]
    st = np.concatenate([s.state(values) for s in fwd])
    np.testing.assert_allclose(st, O.simulate_state(programs, names, values), atol=1e-5)
    smp = np.concatenate([s.samples(values, 50, seed=5) for s in fwd])
    assert smp.shape == (len(programs), 50, 9)
    for i, p in enumerate(programs):
        n = O._parse_all([p], names, values[i:i + 1])[0][0][0]
        assert (smp[i, :, : 9 - n] == -2).all() and (smp[i, :, 9 - n:] >= 0).all()
