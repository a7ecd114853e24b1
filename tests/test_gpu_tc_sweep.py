"""The two-block tensor-core sweep (tc_gates.cu tc_sweep_kernel) on the GPU:
two random 5-qubit unitaries applied to a random state in one pass (tiles
staged by bulk copies, A operands in tensor memory, split 3xTF32), twice in
a row, against numpy in complex128 -- with position 3 of the tile a target
(the staging swizzle on), blocks sharing bits, equal target sets and small
grids (several tiles per CTA, both staging buffers in turn)."""

import numpy as np
import pytest

from quantum_gb300 import _native

pytestmark = pytest.mark.gpu


def _unitary(rng, d=32):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _apply_np(psi, n, tgt, U):
    idx = np.arange(1 << n)
    tmask = sum(1 << t for t in tgt)
    base = idx[(idx & tmask) == 0]
    off = np.array([sum(((j >> i) & 1) << t for i, t in enumerate(tgt)) for j in range(32)])
    pos = base[:, None] + off[None, :]
    out = psi.copy()
    out[pos] = psi[pos] @ U.T
    return out


@pytest.mark.parametrize("n,t0,t1,grid", [
    (14, (4, 5, 6, 7, 8), (9, 10, 11, 12, 13), 0),
    (16, (4, 7, 9, 12, 15), (5, 7, 8, 12, 14), 1),
    (17, (10, 11, 12, 13, 14), (12, 13, 14, 15, 16), 3),
    (15, (4, 5, 6, 7, 8), (4, 5, 6, 7, 8), 2),
    (18, (4, 9, 13, 16, 17), (6, 8, 11, 14, 15), 0),
])
def test_sweep_matches_complex128(n, t0, t1, grid):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(n * 31 + t0[0] + t1[-1])
    U0, U1 = _unitary(rng).astype(np.complex64), _unitary(rng).astype(np.complex64)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi = (psi / np.linalg.norm(psi)).astype(np.complex64)
    tpsi = torch.tensor(psi, device=dev)
    tu0, tu1 = torch.tensor(U0, device=dev), torch.tensor(U1, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream().cuda_stream
    want = psi.astype(np.complex128)
    for _ in range(2):
        _native.tc_sweep(tpsi.data_ptr(), n, tu0.data_ptr(), tu1.data_ptr(), t0, t1,
                         st.data_ptr(), s, grid)
        want = _apply_np(_apply_np(want, n, t0, U0.astype(np.complex128)), n, t1,
                         U1.astype(np.complex128))
    torch.cuda.synchronize()
    assert int(st.item()) == 0, "a bounded wait timed out"
    got = tpsi.cpu().numpy()
    assert np.abs(got - want).max() < 1e-6
