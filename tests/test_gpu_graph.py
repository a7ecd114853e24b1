"""A batch's forward calls captured in CUDA graphs (tfqg_batch_graph_create /
tfqg_graph_launch): an uneven batch -- resident rows, streamed rows in the
queue and lockstep rows of 17-18 qubits -- replayed as one graph launch per
call.  Replays give what direct calls give: expectations and states equal,
samples identical for the captured seed, and new symbol values written into
the captured value buffer are picked up by the next replay."""

import numpy as np
import pytest

from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S
from tests.circuits import random_circuit, random_paulisum

pytestmark = pytest.mark.gpu

NQS = [3, 17, 9, 15, 18, 12, 17]


@pytest.fixture
def batch():
    old = (_native.set_lock_min_qubits(17), _native.set_wide_few_rows(0))
    rng = np.random.default_rng(77)
    names = ["a", "b", "c"]
    programs, psums = [], []
    for n in NQS:
        qs = S.GridQubit.rect(1, n)
        programs.append(S.serialize_circuit(random_circuit(qs, 4, rng, names, p_control=0.2)))
        psums.append([random_paulisum(qs, rng) for _ in range(2)])
    b = ops.Batch(programs, names, psums)
    assert _native.batch_lock_rows(b._h)[0] == 3
    yield b, rng
    b.close()
    _native.set_lock_min_qubits(old[0])
    _native.set_wide_few_rows(old[1])


def test_expectation_graph_follows_new_values(batch):
    import torch
    b, rng = batch
    vals = torch.tensor(rng.uniform(-2, 2, size=(len(NQS), 3)).astype(np.float32),
                        device="cuda:0")
    g = b.capture("expectation", vals)
    try:
        for _ in range(2):
            got = g.replay().clone()
            torch.cuda.synchronize()
            np.testing.assert_array_equal(got.cpu().numpy(), b.expectation(vals).cpu().numpy())
            vals.copy_(torch.tensor(rng.uniform(-2, 2, size=(len(NQS), 3)).astype(np.float32)))
    finally:
        g.close()


def test_samples_and_state_graphs(batch):
    import torch
    b, rng = batch
    vals = torch.tensor(rng.uniform(-2, 2, size=(len(NQS), 3)).astype(np.float32),
                        device="cuda:0")
    gs = b.capture("samples", vals, num_samples=500, seed=4242)
    gt = b.capture("state", vals)
    try:
        for _ in range(2):
            s = gs.replay().clone()
            st = gt.replay().clone()
            torch.cuda.synchronize()
            np.testing.assert_array_equal(s.cpu().numpy(),
                                          b.samples(vals, 500, seed=4242).cpu().numpy())
            np.testing.assert_array_equal(st.cpu().numpy(), b.state(vals).cpu().numpy())
    finally:
        gs.close()
        gt.close()
