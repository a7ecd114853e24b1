"""Sharding a batch across GPUs, one process per GPU.

Circuits (and trajectories) are independent, so a batch splits into
contiguous row ranges, one per rank. Each rank compiles and simulates only
its own rows, and no collective runs on the data path. The outputs are
gathered once at the end, in row order. This is the multi-device form of the
reference's `ParallelFor` over circuits (tfq_simulate_expectation_op.cc:
108-174, tfq_adj_grad_op.cc:173-276), with a device in the role of a
thread-pool shard.

Ranges balance the estimated simulation cost (gates x 2^n per row), not the
row count. In an uneven batch (circuits of 4..20 qubits) one 20-qubit row
costs as much as thousands of small ones.
"""

import ctypes

import numpy as np

from . import _native, ops


def survey(programs, symbol_names):
    """(estimated cost of every row, qubit count of the widest row), from
    a host-side parse of the whole batch (no GPU)."""
    b = ops.Batch(programs, symbol_names, None, kind=ops.KIND_FORWARD)
    n = b.batch_size
    out = (ctypes.c_double * max(n, 1))()
    f = _native.lib().tfqg_internal_batch_row_costs
    f.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    f.restype = ctypes.c_int
    _native.check(f(b._h, out))
    max_n = b.max_num_qubits
    b.close()
    return np.array(out[:n], dtype=np.float64), max_n


def row_costs(programs, symbol_names):
    """Estimated cost of every row (gates x 2^n; 0 for empty programs)."""
    return survey(programs, symbol_names)[0]


def partition(costs, world):
    """Contiguous [start, stop) ranges, one per rank, covering every row.

    Boundary k sits where the cost prefix sum is nearest to k/world of the
    total, so that every range carries about the same work. Ranges may be
    empty when there are fewer rows than ranks."""
    costs = np.asarray(costs, dtype=np.float64)
    n = len(costs)
    if world < 1:
        raise ValueError("world must be >= 1")
    # zero-cost rows (empty programs) still take a little time: weight 1
    w = np.where(costs > 0, costs, 1.0)
    prefix = np.concatenate([[0.0], np.cumsum(w)])
    total = prefix[-1]
    bounds = [0]
    for k in range(1, world):
        target = total * k / world
        j = int(np.searchsorted(prefix, target))
        # nearest prefix point to the target, never before the last boundary
        if j > 0 and (j > n or target - prefix[j - 1] < prefix[j] - target):
            j -= 1
        bounds.append(min(max(j, bounds[-1]), n))
    bounds.append(n)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def gather_rows(local, ranges, group=None):
    """All-gather of per-rank row blocks into the full array on every rank.

    `local` is a torch tensor holding this rank's rows (rows first). With
    NCCL it must be on this rank's GPU; with gloo, on the CPU. Blocks are
    padded to the longest range for the collective and trimmed after it."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    if len(ranges) != world:
        raise ValueError("one range per rank is required")
    longest = max(e - s for s, e in ranges)
    pad = torch.zeros((longest,) + tuple(local.shape[1:]), dtype=local.dtype,
                      device=local.device)
    pad[: local.shape[0]] = local
    blocks = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(blocks, pad, group=group)
    return torch.cat([blk[: e - s] for blk, (s, e) in zip(blocks, ranges)], dim=0)


def _like(x, shape, fill):
    """A new array or tensor of x's kind, dtype and device, filled."""
    if isinstance(x, np.ndarray):
        return np.full(shape, fill, dtype=x.dtype)
    import torch
    return torch.full(shape, fill, dtype=x.dtype, device=x.device)


def widen_states(out, max_n):
    """States of a shard, [rows, 2^local_max_n], padded with -2 to the whole
    batch's 2^max_n columns (tfq_simulate_state_op.cc:201-207)."""
    width = 2 ** max_n
    if out.shape[1] == width:
        return out
    full = _like(out, (out.shape[0], width), -2.0)
    full[:, : out.shape[1]] = out
    return full


def widen_samples(out, max_n):
    """Samples of a shard, [rows, S, local_max_n], widened to max_n columns:
    bit k stays in column max_n - k - 1 and the new leading columns hold -2
    (tfq_simulate_samples_op.cc:227-243)."""
    if out.shape[2] == max_n:
        return out
    full = _like(out, (out.shape[0], out.shape[1], max_n), -2)
    full[:, :, max_n - out.shape[2]:] = out
    return full


class ShardedBatch:
    """This rank's share of a batch, compiled once and run many times.

    Each call takes the full batch's inputs and slices out this rank's rows.
    The returned tensor holds this rank's rows only; pass it to
    `gather_rows(out, self.ranges)` for the whole batch."""

    def __init__(self, programs, symbol_names, pauli_sums=None,
                 kind=ops.KIND_FORWARD, rank=0, world=1):
        programs = list(programs)
        costs, self.max_num_qubits = survey(programs, symbol_names)
        self.ranges = partition(costs, world)
        self.rank = rank
        s, e = self.ranges[rank]
        self.rows = slice(s, e)
        # an object array keeps the [rows, ops] shape of an empty slice
        ps = None
        if pauli_sums is not None:
            ps = np.empty((len(programs), len(pauli_sums[0]) if len(programs) else 0),
                          dtype=object)
            for i, r in enumerate(pauli_sums):
                for j, x in enumerate(r):
                    ps[i, j] = x
            ps = ps[s:e]
        self.local = ops.Batch(programs[s:e], symbol_names, ps, kind=kind)

    def expectation(self, symbol_values):
        return self.local.expectation(symbol_values[self.rows])

    def adj_grad(self, symbol_values, downstream_grads, grad_rule=ops.GRAD_REFERENCE_FD):
        return self.local.adj_grad(symbol_values[self.rows],
                                   downstream_grads[self.rows], grad_rule)

    def state(self, symbol_values):
        return widen_states(self.local.state(symbol_values[self.rows]),
                            self.max_num_qubits)

    def samples(self, symbol_values, num_samples, seed=None):
        if seed is not None:  # a distinct random stream per rank
            seed = (int(seed) + 0x9E3779B97F4A7C15 * self.rank) & (2 ** 64 - 1)
        out = self.local.samples(symbol_values[self.rows], num_samples, seed)
        return widen_samples(out, self.max_num_qubits)

    def noisy_expectation(self, symbol_values, num_samples, seed=None):
        if seed is not None:
            seed = (int(seed) + 0x9E3779B97F4A7C15 * self.rank) & (2 ** 64 - 1)
        return self.local.noisy_expectation(symbol_values[self.rows],
                                            num_samples[self.rows], seed)
