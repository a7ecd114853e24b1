"""The multi-GPU form of the path on CPU: batches split into cost-balanced
contiguous row ranges, one per rank, with no collective on the data path, and
outputs gathered in row order. Two `gloo` ranks run as child processes. The
oracle computes each rank's rows here, since these ranks have no GPU. The
gathered result must equal the oracle over the whole batch."""

import os
import socket

import numpy as np
import pytest

from oracle import tfq_oracle as O
from quantum_gb300 import ops, sharding
from quantum_gb300 import serialize as S
from tests.circuits import random_circuit, random_paulisum


def _uneven(seed=3, sizes=(2, 9, 3, 3, 8, 1, 4, 2, 7)):
    rng = np.random.default_rng(seed)
    names = ["a", "b", "c"]
    programs, psums = [], []
    for n in sizes:
        qs = S.GridQubit.rect(1, n)
        programs.append(S.serialize_circuit(random_circuit(qs, 4, rng, names)))
        psums.append([random_paulisum(qs, rng), random_paulisum(qs, rng)])
    programs.append(S.serialize_circuit(S.Circuit([])))  # empty program
    psums.append([S.serialize_paulisum([]), S.serialize_paulisum([])])
    values = rng.uniform(-1, 1, size=(len(programs), len(names))).astype(np.float32)
    return programs, names, values, psums


def test_partition_covers_and_balances():
    rng = np.random.default_rng(0)
    for world in (1, 2, 3, 8):
        costs = rng.integers(1, 2 ** 12, size=50).astype(float)
        r = sharding.partition(costs, world)
        assert r[0][0] == 0 and r[-1][1] == 50
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
        loads = [costs[s:e].sum() for s, e in r]
        # no range exceeds its share by more than one row's cost
        assert max(loads) <= costs.sum() / world + costs.max()
    assert sharding.partition([5.0], 3) == [(0, 0), (0, 1), (1, 1)]
    assert sharding.partition([], 2) == [(0, 0), (0, 0)]


def test_row_costs_follow_width_and_depth():
    programs, names, _, _ = _uneven()
    costs = sharding.row_costs(programs, names)
    assert costs[-1] == 0.0  # empty program
    assert costs[1] > costs[4] > costs[0]  # 9 qubits > 8 qubits > 2 qubits


def test_widen_states_and_samples_match_whole_batch_layout():
    programs, names, values, _ = _uneven()
    whole = O.simulate_state(programs, names, values)
    for s, e in [(0, 3), (3, 6), (6, 10)]:
        part = O.simulate_state(programs[s:e], names, values[s:e])
        np.testing.assert_array_equal(sharding.widen_states(part, 9), whole[s:e])
    idx = np.arange(16)
    local = O.sample_bits_layout(idx, 3, 4)[None]
    np.testing.assert_array_equal(sharding.widen_samples(local, 9)[0],
                                  O.sample_bits_layout(idx, 3, 9))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        programs, names, values, psums = _uneven()
        dg = np.linspace(-1, 1, 2 * len(programs)).reshape(-1, 2).astype(np.float32)
        sb = sharding.ShardedBatch(programs, names, psums, kind=ops.KIND_ADJOINT,
                                   rank=rank, world=world)
        s, e = sb.ranges[rank]
        assert sb.local.batch_size == e - s
        # every rank derives the same ranges from the same inputs
        all_ranges = [None] * world
        dist.all_gather_object(all_ranges, sb.ranges)
        assert all(r == sb.ranges for r in all_ranges)
        exp = O.simulate_expectation(programs[s:e], names, values[s:e], psums[s:e])
        grad = O.adj_grad(programs[s:e], names, values[s:e], psums[s:e], dg[s:e])
        st = sharding.widen_states(
            O.simulate_state(programs[s:e], names, values[s:e]), sb.max_num_qubits)
        full_exp = sharding.gather_rows(torch.from_numpy(np.asarray(exp, np.float64)),
                                        sb.ranges)
        full_grad = sharding.gather_rows(torch.from_numpy(np.asarray(grad, np.float64)),
                                         sb.ranges)
        full_st = sharding.gather_rows(torch.from_numpy(st), sb.ranges)
        if rank == 0:
            q.put((full_exp.numpy(), full_grad.numpy(), full_st.numpy(),
                   [e - s for s, e in sb.ranges]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_the_whole_batch():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got_exp, got_grad, got_st, sizes = q.get(timeout=240)
    finally:
        for p in procs:
            p.join(timeout=60)
    assert all(p.exitcode == 0 for p in procs)
    assert min(sizes) > 0  # both ranks did work
    programs, names, values, psums = _uneven()
    dg = np.linspace(-1, 1, 2 * len(programs)).reshape(-1, 2).astype(np.float32)
    np.testing.assert_allclose(got_exp, O.simulate_expectation(programs, names, values, psums),
                               atol=1e-12)
    np.testing.assert_allclose(got_grad, O.adj_grad(programs, names, values, psums, dg),
                               atol=1e-12)
    np.testing.assert_allclose(got_st, O.simulate_state(programs, names, values), atol=1e-12)
