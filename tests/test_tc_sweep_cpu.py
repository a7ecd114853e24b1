"""Index arithmetic of the two-block tensor-core sweep (tc_gates.cu
tc_sweep_kernel), restated on the CPU from the geometry the library computes
for the launch (tfqg_internal_tc_sweep_geometry), before it runs on a GPU:

- the tile holds 13 index bits: bits 0-2, both blocks' targets and the
  lowest free bits; bulk copies move runs of 2^r0 amplitudes that are
  contiguous both in the state and in the swizzled staging buffer, and the
  swizzle is a bijection on the tile's 8192 slots;
- for each block, (group, amplitude j) covers the tile once, and the 32
  amplitudes of a group differ exactly in the block's target bits, j's bit i
  on target i;
- the tiles' bases are distinct and avoid the tile bits;
- the 32 lanes of a warp reading amplitude j of their groups hit 16
  distinct 8-byte bank slots, twice each."""

import ctypes

import numpy as np
import pytest

from quantum_gb300 import _native, ops, workloads


def _geometry(n, t0, t1):
    f = _native.lib().tfqg_internal_tc_sweep_geometry
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    a, b = (ctypes.c_int32 * 5)(*t0), (ctypes.c_int32 * 5)(*t1)
    out = (ctypes.c_uint32 * 10)()
    ok = f(n, a, b, out)
    return ok, list(out)


def _check(n, t0, t1):
    ok, v = _geometry(n, t0, t1)
    if min(t0) < 4 or min(t1) < 4:
        assert not ok
        return False
    assert ok
    cb = v[0] | (v[1] << 32)
    CB = [(cb >> (5 * p)) & 31 for p in range(12)] + [v[2]]
    smask, hmask, r0 = v[3], v[8], v[9]
    assert CB == sorted(CB) and len(set(CB)) == 13 and set(range(3)) <= set(CB)
    assert sum(1 << b for b in CB) == smask and set(t0) | set(t1) <= set(CB)
    assert CB[:r0] == list(range(r0)) and r0 >= 3

    def dep(L):
        return sum(1 << CB[p] for p in range(13) if (L >> p) & 1)

    def slot(L):
        return L ^ ((bin(L & hmask).count("1") & 1) << 3)

    sl = np.array([slot(L) for L in range(8192)])
    assert sorted(sl) == list(range(8192))
    run = 1 << r0
    for q in range(0, 8192 >> r0, 7):
        L0 = q << r0
        assert all(dep(L0 + i) == dep(L0) + i for i in range(run))
        assert all(slot(L0 + i) == slot(L0) + i for i in range(run))
    for b, tg in enumerate((t0, t1)):
        tpos = [(v[4 + b] >> (4 * i)) & 15 for i in range(5)]
        rpos = [(v[6 + b] >> (4 * i)) & 15 for i in range(8)]
        assert [CB[p] for p in tpos] == list(tg)
        assert sorted(tpos + rpos) == list(range(13))

        def deposit(x, pos):
            return sum(1 << pos[i] for i in range(len(pos)) if (x >> i) & 1)
        seen = set()
        for gi in range(256):
            Lr = deposit(gi, rpos)
            for j in range(32):
                L = Lr | deposit(j, tpos)
                seen.add(L)
                assert dep(L) - dep(Lr) == sum(((j >> i) & 1) << tg[i] for i in range(5))
        assert len(seen) == 8192
        for w in range(8):
            for j in range(32):
                s = [slot(deposit((w >> 2) * 128 + (w & 3) * 32 + l, rpos) |
                          deposit(j, tpos)) & 15 for l in range(32)]
                assert sorted(np.bincount(s, minlength=16)) == [2] * 16
    outside = [b for b in range(n) if not (smask >> b) & 1]
    bases = set()
    for t in list(range(min(1 << (n - 13), 64))) + [(1 << (n - 13)) - 1]:
        base = sum(1 << outside[k] for k in range(len(outside)) if (t >> k) & 1)
        assert base & smask == 0
        bases.add(base)
    assert len(bases) == len(set(list(range(min(1 << (n - 13), 64))) + [(1 << (n - 13)) - 1]))
    return True


def test_consecutive_blocks_of_the_30_qubit_plan():
    w = workloads.grid_fsim(5, 6, 24, seed=1)
    b = ops.Batch(w["programs"], [], w["pauli_sums"])
    plan = [tuple(int(t) for t in p[0])
            for p in _native.tc_plan(b._h, 0, np.zeros(0, np.float32))]
    b.close()
    paired = sum(_check(30, plan[i], plan[i + 1]) for i in range(len(plan) - 1))
    assert paired > 10


@pytest.mark.parametrize("n", [14, 17, 22])
def test_random_pairs(n):
    rng = np.random.default_rng(n)
    for _ in range(10):
        t0 = tuple(sorted(int(x) for x in rng.choice(range(4, n), 5, replace=False)))
        t1 = tuple(sorted(int(x) for x in rng.choice(range(4, n), 5, replace=False)))
        _check(n, t0, t1)
    _check(n, (4, 5, 6, 7, 8), (9, 10, 11, 12, 13))  # position 3 a target, no bit 3
    _check(n, (4, 5, 6, 7, 8), (4, 5, 6, 7, 8))
    assert not _check(n, (3, 5, 6, 7, 8), (9, 10, 11, 12, 13))
