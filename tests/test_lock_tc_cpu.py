"""The schedule of lockstep rows on tensor-core blocks, built on the host when
a batch is created (no GPU): every lockstep row with a 5-qubit plan
contributes its plan's blocks; launch q of a variant (direct, or transposed
for blocks with a target below bit 5) covers block q of every such row, in
units of up to 16 chunks of 128 groups, fewer when the launch would have
under 256 units; the default (blocks from 15 qubits), the
per-qubit-count policy (2: tensor-core blocks, 1: tile passes) and the
tensor-core switch decide which rows take them; a row whose gate spans six bits keeps its tile passes."""

import numpy as np

from quantum_gb300 import _native, autotune, ops
from quantum_gb300 import serialize as S
from tests.circuits import make_gate, random_circuit


def _programs(nqs, seed=0, six_bit_row=None):
    rng = np.random.default_rng(seed)
    out = []
    for r, n in enumerate(nqs):
        qs = S.GridQubit.rect(1, n)
        c = random_circuit(qs, 6, rng, [])
        if r == six_bit_row:
            op = make_gate(rng, "CZP", [qs[1], qs[n - 2]], [], 0.0)
            c.moments.insert(0, [op.controlled_by(qs[0], qs[3], qs[6], qs[n - 1])])
        out.append(S.serialize_circuit(c))
    return out


class _Settings:
    def __enter__(self):
        self.old = (_native.set_lock_min_qubits(14), _native.set_wide_few_rows(0),
                    _native.set_lock_tc(True), _native.set_tensor_core_gates(2))
        autotune.reset()
        return self

    def __exit__(self, *exc):
        _native.set_lock_min_qubits(self.old[0])
        _native.set_wide_few_rows(self.old[1])
        _native.set_lock_tc(self.old[2])
        _native.set_tensor_core_gates(self.old[3])
        autotune.reset()


def _expected(b, nqs, rows):
    plans = {r: _native.tc_plan(b._h, r, np.zeros(0, np.float32)) for r in rows}
    assert all(p is not None for p in plans.values())
    blocks = sum(len(p) for p in plans.values())
    units = 0
    for q in range(max(len(p) for p in plans.values())):
        for trans in (False, True):
            chunks = [2 ** (nqs[r] - 12) for r, p in plans.items()
                      if q < len(p) and (p[q][0][0] < 5) == trans]
            per = 16
            while per > 1 and sum(chunks) // per < 256:
                per //= 2
            units += sum(-(-c // per) for c in chunks)
    return blocks, units


def test_units_follow_the_plans():
    nqs = [15, 18, 6, 17, 21, 15]
    progs = _programs(nqs)
    with _Settings():
        b = ops.Batch(progs, [], None)
        assert _native.batch_lock_rows(b._h)[0] == 5
        assert _native.batch_lock_tc(b._h) == _expected(b, nqs, [0, 1, 3, 4, 5])


def test_default_and_policy_choose_the_rows():
    nqs = [16, 18, 18, 16]
    progs = _programs(nqs, seed=1)
    with _Settings():
        _native.set_lock_tc(False)
        b = ops.Batch(progs, [], None)
        assert _native.batch_lock_rows(b._h)[0] == 4
        assert _native.batch_lock_tc(b._h) == (0, 0)
        autotune.set_row_policy(18, lock=2)
        b = ops.Batch(progs, [], None)
        assert _native.batch_lock_tc(b._h) == _expected(b, nqs, [1, 2])
        _native.set_lock_tc(True)
        autotune.set_row_policy(18, lock=1)
        b = ops.Batch(progs, [], None)
        assert _native.batch_lock_tc(b._h) == _expected(b, nqs, [0, 3])
        autotune.reset()
        _native.set_lock_tc(2)  # the default: blocks from 15 qubits
        b = ops.Batch(progs, [], None)
        assert _native.batch_lock_tc(b._h) == _expected(b, nqs, [0, 1, 2, 3])
        _native.set_tensor_core_gates(0)
        b = ops.Batch(progs, [], None)
        assert _native.batch_lock_rows(b._h)[0] == 4
        assert _native.batch_lock_tc(b._h) == (0, 0)


def test_row_without_plan_keeps_tile_passes():
    nqs = [16, 17, 16]
    progs = _programs(nqs, seed=2, six_bit_row=1)
    with _Settings():
        b = ops.Batch(progs, [], None)
        assert _native.batch_lock_rows(b._h)[0] == 3
        assert _native.tc_plan(b._h, 1, np.zeros(0, np.float32)) is None
        assert _native.batch_lock_tc(b._h) == _expected(b, nqs, [0, 2])


def test_persistent_queue_order():
    """The persistent form's queue: per row, units of one block after
    another (every chunk once per block); a unit needs exactly its row's
    units of earlier blocks, and all of them come before it in the queue (so
    a waiting unit never waits on one not yet taken)."""
    nqs = [15, 18, 6, 17, 20, 16]
    progs = _programs(nqs, seed=3)
    with _Settings():
        old = _native.set_lock_arena_amps(1 << 19)  # several groups
        try:
            b = ops.Batch(progs, [], None)
        finally:
            _native.set_lock_arena_amps(old)
        pu = _native.batch_lock_punits(b._h)
        lock = [r for r, n in enumerate(nqs) if n >= 15]
        blocks = {r: len(_native.tc_plan(b._h, r, np.zeros(0, np.float32))) for r in lock}
        assert len(np.unique(pu[:, 0])) > 1
        seen, row_of = {}, {}
        for g, slot, row, need, c0, nch in pu:
            assert row_of.setdefault(slot, row) == row
            prev = seen.setdefault(slot, [])
            # the units this one needs: its row's units of earlier blocks,
            # all already in the queue
            assert need == sum(1 for (nd, _, _) in prev if nd < need) <= len(prev)
            prev.append((need, c0, nch))
        # every row: each of its blocks covers each of its chunks once
        assert sorted(row_of.values()) == lock
        for slot, r in row_of.items():
            chunks = 2 ** (nqs[r] - 12)
            assert len({need for need, _, _ in seen[slot]}) == blocks[r]
            cover = {}
            for need, c0, nch in seen[slot]:
                cover.setdefault(need, []).extend(range(c0, c0 + nch))
            assert all(sorted(v) == list(range(chunks)) for v in cover.values())
