"""The process-wide cache of compiled and planned programs (host only).

A batch built from cached programs must have the same packed tables as one
built from scratch; the key must cover the symbol-name order, the job kind
and the fusion setting; invalid programs are never cached, so their errors
repeat; the cache stays within its capacity, evicting the least recently
used entries, and a batch that fits hits on every program the second time;
the tensor-core block plan kept in an entry gives the lockstep schedule
that planning from scratch gives."""

import numpy as np
import pytest

from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S
from tests.circuits import random_circuit, random_paulisum


def _inputs(seed=3, nqs=(3, 6, 9, 14, 16)):
    rng = np.random.default_rng(seed)
    names = ["a", "b", "c"]
    programs, psums = [], []
    for n in nqs:
        qs = S.GridQubit.rect(1, n)
        programs.append(S.serialize_circuit(random_circuit(qs, 6, rng, names, p_control=0.3)))
        psums.append([random_paulisum(qs, rng)])
    return programs, names, psums


@pytest.fixture
def fresh_cache():
    _native.program_cache(False)  # empties it
    _native.program_cache(True)
    yield
    _native.program_cache(True)


def _fp(programs, names, psums, kind):
    b = ops.Batch(programs, names, psums, kind=kind)
    fp = _native.batch_fingerprint(b._h)
    b.close()
    return fp


@pytest.mark.parametrize("kind", [ops.KIND_FORWARD, ops.KIND_ADJOINT])
def test_cached_batch_has_identical_tables(fresh_cache, kind):
    programs, names, psums = _inputs()
    _, h0, m0 = _native.program_cache()
    first = _fp(programs, names, psums, kind)
    _, h1, m1 = _native.program_cache()
    second = _fp(programs, names, psums, kind)
    _, h2, m2 = _native.program_cache()
    assert m1 - m0 == len(programs) and h1 == h0
    assert h2 - h1 == len(programs) and m2 == m1
    assert first == second
    _native.program_cache(False)
    assert _fp(programs, names, psums, kind) == first
    _native.program_cache(True)


def test_key_covers_names_kind_and_fusion(fresh_cache):
    programs, names, psums = _inputs(seed=4)
    base = _fp(programs, names, psums, ops.KIND_FORWARD)
    _, h0, _ = _native.program_cache()
    # the same names in another order bind symbols to other columns
    _fp(programs, names[::-1], psums, ops.KIND_FORWARD)
    _fp(programs, names, psums, ops.KIND_ADJOINT)
    prev = _native.set_gate_fusion(False)
    try:
        unfused = _fp(programs, names, psums, ops.KIND_FORWARD)
    finally:
        _native.set_gate_fusion(prev)
    _, h1, _ = _native.program_cache()
    assert h1 == h0, "a changed key must not hit"
    assert unfused != base
    # and each of them is reused on its own key
    assert _fp(programs, names, psums, ops.KIND_FORWARD) == base


def test_invalid_programs_are_not_cached(fresh_cache):
    q = S.GridQubit.rect(1, 2)
    bad = S.serialize_circuit(S.Circuit([[S.rx(q[0], S.Symbol("missing"))], [S.I(q[1])]]))
    for _ in range(2):
        with pytest.raises(_native.InvalidArgumentError):
            ops.Batch([bad], ["a"], None)


def test_empty_program_cached_keeps_its_semantics(fresh_cache):
    empty = S.serialize_circuit(S.Circuit([]))
    q = S.GridQubit.rect(1, 2)
    ps = S.serialize_paulisum([(1.0, [(q[0], "Z")])])
    fps = {_fp([empty], [], [[ps]], ops.KIND_FORWARD) for _ in range(2)}
    assert len(fps) == 1


def test_capacity_and_eviction(fresh_cache):
    programs, names, psums = _inputs(seed=5, nqs=tuple(range(3, 15)) * 3)
    old = _native.program_cache_capacity(1 << 16)
    try:
        b = ops.Batch(programs, names, psums)
        b.close()
        n, nbytes = _native.program_cache_size()
        assert 0 < n < len(programs) and nbytes <= 1 << 16, (n, nbytes)
        _native.program_cache_capacity(1 << 30)
        b = ops.Batch(programs, names, psums)
        b.close()
        _, h0, m0 = _native.program_cache()
        b = ops.Batch(programs, names, psums)
        b.close()
        _, h1, m1 = _native.program_cache()
        assert (h1 - h0, m1 - m0) == (len(programs), 0)
    finally:
        _native.program_cache_capacity(old)


def test_cached_tensor_core_plans_give_the_same_schedule(fresh_cache):
    programs, names, psums = _inputs(seed=7, nqs=(15, 16, 17, 15))
    old = (_native.set_lock_min_qubits(15), _native.set_wide_few_rows(0), _native.set_lock_tc(1))
    try:
        first = ops.Batch(programs, names, psums)   # plans, keeps them in the cache
        again = ops.Batch(programs, names, psums)   # takes them from the cache
        _native.program_cache(False)
        fresh = ops.Batch(programs, names, psums)   # plans without a cache
        want = _native.batch_lock_tc(fresh._h)
        assert want[0] > 0
        for b in (first, again):
            assert _native.batch_lock_tc(b._h) == want
            np.testing.assert_array_equal(_native.batch_lock_punits(b._h),
                                          _native.batch_lock_punits(fresh._h))
        for b in (first, again, fresh):
            b.close()
    finally:
        _native.set_lock_min_qubits(old[0])
        _native.set_wide_few_rows(old[1])
        _native.set_lock_tc(old[2])
