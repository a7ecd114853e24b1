"""Index arithmetic of the tensor-core block kernel's transposed variant
(quantum_gb300/csrc/tc_gates.cu, blocks with a target among bits 0-4),
restated on the CPU from the geometry the library computes for the launch
(tfqg_internal_tc_geometry), before any of it runs on a GPU:

- every (group row, amplitude j) that a thread reads from the staging buffer
  is the amplitude the direct variant would gather for that group: the same
  global index, so the transposed variant applies the block to the same
  groups;
- the swizzle is a bijection on the 4096 staging slots, keeps the two
  amplitudes of a 16-byte vector in one 16-byte unit, and every global
  access stays inside the 2^n state;
- no bank conflicts beyond the minimum: the 32 lanes of a warp reading
  amplitude j of their groups (8-byte accesses) hit 16 distinct bank pairs,
  twice each, and 8 consecutive lanes of the 16-byte linear accesses hit 8
  distinct 16-byte units."""

import ctypes

import numpy as np
import pytest

from quantum_gb300 import _native, ops, workloads


def _geometry(n, tgt):
    f = _native.lib().tfqg_internal_tc_geometry
    f.argtypes = [ctypes.c_int, ctypes.c_void_p] + [ctypes.c_void_p] * 4
    f.restype = ctypes.c_int
    t = (ctypes.c_int32 * 5)(*tgt)
    cb, rpos, tpos, c = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
    ok = f(n, t, ctypes.byref(cb), ctypes.byref(rpos), ctypes.byref(tpos), ctypes.byref(c))
    return ok, cb.value, rpos.value, tpos.value, c.value


def _group_base(g, t):
    for ti in t:
        low = (1 << ti) - 1
        g = ((g & ~low) << 1) | (g & low)
    return g


def _check(n, tgt, rng):
    ok, cb, rpos, tpos, c = _geometry(n, tgt)
    assert ok == (tgt[0] < 5)
    if not ok:
        return
    CB = [(cb >> (5 * p)) & 31 for p in range(12)]
    RP = [(rpos >> (4 * i)) & 15 for i in range(7)]
    TP = [(tpos >> (4 * i)) & 15 for i in range(5)]
    C = [(c >> (4 * i)) & 15 for i in range(8)]
    assert sorted(RP + TP) == list(range(12))
    assert CB == sorted(CB) and set(range(7)) <= set(CB) and max(CB) < n
    assert [CB[p] for p in TP] == list(tgt)

    def dep(L):
        return sum(1 << CB[p] for p in range(12) if (L >> p) & 1)

    def h(L):
        x = 0
        for p in range(4, 12):
            if (L >> p) & 1:
                x ^= C[p - 4]
        return x

    def deposit(v, pos, bits):
        return sum(1 << pos[i] for i in range(bits) if (v >> i) & 1)

    sw = np.array([L ^ h(L) for L in range(4096)])
    assert sorted(sw) == list(range(4096))                   # bijection
    assert all((sw[L] >> 1) == (sw[L + 1] >> 1) for L in range(0, 4096, 2))
    nchunk = 1 << (n - 12)
    direct_off = [sum(((j >> i) & 1) << tgt[i] for i in range(5)) for j in range(32)]
    for ch in {0, nchunk - 1, int(rng.integers(nchunk))}:
        base = _group_base(ch * 128, tgt)
        for r in range(128):
            Lr = deposit(r, RP, 7)
            gb = _group_base(ch * 128 + r, tgt)
            for j in range(32):
                L = Lr | deposit(j, TP, 5)
                assert base + dep(L) == gb + direct_off[j]
        assert base + dep(4095) < (1 << n)
    # bank pairs of the 8-byte row accesses: lanes r = 32 w + l, amplitude j
    for w in range(4):
        for j in range(32):
            slots = [sw[deposit(32 * w + l, RP, 7) | deposit(j, TP, 5)] & 15 for l in range(32)]
            assert sorted(np.bincount(slots, minlength=16)) == [2] * 16
    # 16-byte linear accesses: lanes 8q..8q+7 of L = 2 t + 256 i
    for i in range(16):
        for t0 in range(0, 128, 8):
            units = [(sw[2 * t + 256 * i] >> 1) & 7 for t in range(t0, t0 + 8)]
            assert len(set(units)) == 8


def test_plan_target_sets_of_the_30_qubit_grid_circuit():
    rng = np.random.default_rng(0)
    w = workloads.grid_fsim(5, 6, 24, seed=1)
    b = ops.Batch(w["programs"], [], w["pauli_sums"])
    sets = {tuple(int(t) for t in p[0])
            for p in _native.tc_plan(b._h, 0, np.zeros(0, np.float32))}
    b.close()
    for tgt in sorted(sets):
        _check(30, tgt, rng)


@pytest.mark.parametrize("n", [12, 13, 17, 24])
def test_random_low_target_sets(n):
    rng = np.random.default_rng(n)
    for _ in range(12):
        low = int(rng.integers(0, 5))
        rest = rng.choice([b for b in range(n) if b != low], size=4, replace=False)
        _check(n, tuple(sorted([low] + [int(x) for x in rest])), rng)
    _check(n, (0, 1, 2, 3, 4), rng)
    _check(n, tuple(range(n - 5, n)), rng)
