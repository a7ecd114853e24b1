"""The allocation-free expectation entry point (tfqg_batch_expectation_noalloc).

Some callers cannot let this library call cudaMalloc, typically a host
framework whose caching allocator has already reserved nearly all device
memory.  The no-allocation entry point keeps all of its scratch in one fixed
device array; this test checks, through the C ABI, that it returns what the
regular entry point returns on a batch that needs that scratch (a 15-qubit
row is streamed through per-CTA state slots), on two calls in a row.

This file is collected last on purpose so that a run stopping at the first
failure has already run every other test."""

import ctypes

import numpy as np
import pytest

from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S
from tests.circuits import random_circuit, random_paulisum

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_entry_point():
    import torch
    lib = _native.lib()
    rng = np.random.default_rng(2024)
    names = [f"s{i}" for i in range(4)]
    programs, psums = [], []
    for n in (15, 5, 9, 15):
        qs = S.GridQubit.rect(1, n)
        programs.append(S.serialize_circuit(random_circuit(qs, 6, rng, names)))
        psums.append([random_paulisum(qs, rng) for _ in range(2)])
    batch = ops.Batch(programs, names, psums, ops.KIND_FORWARD)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        vals = torch.tensor(rng.uniform(-2, 2, size=(4, 4)).astype(np.float32),
                            device=dev)
        want = batch.expectation(vals)
        got = torch.full((4, 2), float("nan"), device=dev)
        rc = lib.tfqg_batch_expectation_noalloc(
            batch._h, ctypes.c_void_p(vals.data_ptr()),
            ctypes.c_void_p(got.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        _native.check(rc)
        torch.cuda.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(),
                                   atol=1e-5 * 8, rtol=0)
