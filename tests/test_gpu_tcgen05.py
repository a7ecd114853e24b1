"""The tcgen05 building blocks (tc_mma.cu) on the GPU: TMEM allocation, the
shared-memory operand and instruction descriptors of a kind::tf32 MMA, its
completion on an mbarrier and the TMEM read-back, as one 128 x 64 x 32 GEMM,
with the A operand in shared memory or in tensor memory (stored there with
tcgen05.st).
Inputs are multiples of 1/8 below 8 in magnitude: exact in tf32, so the
tensor-core result must equal the float64 product exactly."""

import ctypes

import numpy as np
import pytest

from quantum_gb300 import _native

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("entry", ["tfqg_internal_tc_gemm_tf32",
                                   "tfqg_internal_tc_gemm_tf32_ts"])
def test_tc_gemm_tf32_exact_on_tf32_inputs(entry):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(7)
    a = (rng.integers(-63, 64, size=(128, 32)) / 8.0).astype(np.float32)
    b = (rng.integers(-63, 64, size=(64, 32)) / 8.0).astype(np.float32)
    ta, tb = torch.tensor(a, device=dev), torch.tensor(b, device=dev)
    td = torch.full((128, 64), float("nan"), device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    f = getattr(_native.lib(), entry)
    f.argtypes = [ctypes.c_void_p] * 5
    f.restype = ctypes.c_int
    rc = f(ta.data_ptr(), tb.data_ptr(), td.data_ptr(), st.data_ptr(),
           torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == 0
    assert int(st.item()) == 0, "MMA completion wait timed out"
    want = a.astype(np.float64) @ b.astype(np.float64).T
    np.testing.assert_array_equal(td.cpu().numpy(), want.astype(np.float32))
