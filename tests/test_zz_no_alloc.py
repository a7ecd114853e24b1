"""The allocation-free expectation entry point (tfqg_batch_expectation_noalloc).

Some callers cannot let this library call cudaMalloc, typically a host
framework whose caching allocator has already reserved nearly all device
memory.  The no-allocation entry point keeps all of its scratch in one fixed
device array.  These tests check, through the C ABI, that it returns what
the regular entry point returns, on two calls in a row:
- a batch whose 15-qubit rows stream through per-CTA state slots;
- a batch with 20-qubit rows (8 MiB slots: fewer fit in the array than the
  kernel's usual grid, so the grid shrinks; the regular entry point runs
  these rows on the whole GPU) and an empty program (-2);
and that it allocates nothing (free device memory unchanged across calls),
and that a 23-qubit row, whose state slot cannot fit beside the tables, is
refused with RESOURCE_EXHAUSTED.

This file is collected last on purpose so that a run stopping at the first
failure has already run every other test."""

import ctypes

import numpy as np
import pytest

from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S
from tests.circuits import expectation_atol, random_circuit, random_paulisum

pytestmark = pytest.mark.gpu


def _noalloc(batch, vals, out, stream):
    return _native.lib().tfqg_batch_expectation_noalloc(
        batch._h, ctypes.c_void_p(vals.data_ptr()), ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(stream.cuda_stream))


def _inputs(rng, nqs, names, n_moments=6):
    programs, psums = [], []
    for n in nqs:
        if n == 0:
            programs.append(S.serialize_circuit(S.Circuit()))
            qs = S.GridQubit.rect(1, 2)
        else:
            qs = S.GridQubit.rect(1, n)
            programs.append(S.serialize_circuit(random_circuit(qs, n_moments, rng, names)))
        psums.append([random_paulisum(qs, rng) for _ in range(2)] if n else
                     [S.serialize_paulisum([(1.0, [(qs[0], "Z")])])] * 2)
    return programs, psums


@pytest.mark.parametrize("nqs", [(15, 5, 9, 15), (20, 6, 20, 0, 20, 12, 20, 20, 20, 20)])
def test_noalloc_matches_regular_entry_point(nqs):
    import torch
    rng = np.random.default_rng(2024 + len(nqs))
    names = [f"s{i}" for i in range(4)]
    programs, psums = _inputs(rng, nqs, names, n_moments=6 if max(nqs) < 20 else 3)
    batch = ops.Batch(programs, names, psums, ops.KIND_FORWARD)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    B = len(nqs)
    got = torch.full((B, 2), float("nan"), device=dev)
    for call in range(2):
        vals = torch.tensor(rng.uniform(-2, 2, size=(B, 4)).astype(np.float32), device=dev)
        want = batch.expectation(vals)
        got.fill_(float("nan"))
        _native.check(_noalloc(batch, vals, got, stream))
        torch.cuda.synchronize()
        g = got.cpu().numpy()
        np.testing.assert_allclose(g, want.cpu().numpy(), atol=expectation_atol(psums), rtol=0)
        for i, n in enumerate(nqs):
            if n == 0:
                assert (g[i] == -2).all()


def test_noalloc_allocates_nothing():
    """After a first call (device set-up and lazily loaded kernels), further
    calls leave the device's free memory unchanged."""
    import torch
    rng = np.random.default_rng(7)
    names = ["a", "b"]
    programs, psums = _inputs(rng, (16, 8, 18), names)
    batch = ops.Batch(programs, names, psums, ops.KIND_FORWARD)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    vals = torch.tensor(rng.uniform(-2, 2, size=(3, 2)).astype(np.float32), device=dev)
    out = torch.empty((3, 2), device=dev)
    _native.check(_noalloc(batch, vals, out, stream))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    for _ in range(3):
        _native.check(_noalloc(batch, vals, out, stream))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0, (free0, free1)


def test_noalloc_refuses_a_row_whose_slot_cannot_fit():
    import torch
    rng = np.random.default_rng(23)
    programs, psums = _inputs(rng, (23, 4), [], n_moments=1)
    batch = ops.Batch(programs, [], psums, ops.KIND_FORWARD)
    dev = torch.device("cuda", 0)
    vals = torch.zeros((2, 0), device=dev)
    out = torch.empty((2, 2), device=dev)
    rc = _noalloc(batch, vals, out, torch.cuda.current_stream(dev))
    assert rc == 8  # RESOURCE_EXHAUSTED
    with pytest.raises(_native.ResourceExhaustedError, match="scratch"):
        _native.check(rc)
