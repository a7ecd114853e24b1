"""Run-time specialization without a GPU: for batches that exercise every op
form (one- and two-qubit gates of each structure class, register and
non-register controls, channels), the generated per-mode source compiles
with NVRTC for sm_103a.  Loading and running it is covered by the GPU tests
in test_gpu_specialization.py."""

import numpy as np
import pytest

from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S
from tests.circuits import CHANNELS, random_circuit, random_paulisum


def _batch(kind, nqs, channels=()):
    rng = np.random.default_rng(11 + kind)
    names = ["a", "b", "c"]
    programs, psums = [], []
    for n in nqs:
        qs = S.GridQubit.rect(1, n)
        c = random_circuit(qs, 8, rng, names, p_control=0.4,
                           channels=list(channels), p_channel=0.3 if channels else 0)
        programs.append(S.serialize_circuit(c))
        psums.append([random_paulisum(qs, rng)])
    return ops.Batch(programs, names, psums, kind=kind)


@pytest.mark.parametrize("kind,modes", [
    (ops.KIND_FORWARD, ["expect", "state", "sample", "wide"]),
    (ops.KIND_ADJOINT, ["expect", "adjoint"]),
])
def test_generated_source_compiles(kind, modes):
    b = _batch(kind, [5, 9, 16])
    nsig, active, _ = _native.batch_specialization(b._h)
    assert nsig > 0 and not active
    for m in modes:
        _native.specialization_compile_check(b._h, m)


def test_generated_noisy_source_compiles():
    b = _batch(ops.KIND_NOISY, [4, 7], channels=CHANNELS)
    _native.specialization_compile_check(b._h, "noisy")
