"""The one-shot C entry points with HOST buffers (what a TF CPU-side
OpKernel::Compute holds), called through ctypes exactly as a foreign binding
would, against the complex128 oracle: tfqg_simulate_expectation,
tfqg_simulate_state (with tfqg_max_num_qubits sizing the output),
tfqg_simulate_samples, tfqg_adj_grad, tfqg_noisy_expectation,
tfqg_simulate_sampled_expectation and tfqg_inner_product.  Tolerances as in
test_gpu_parity.py."""

import ctypes

import numpy as np
import pytest

from oracle import tfq_oracle as O
from quantum_gb300 import _native
from quantum_gb300 import serialize as S
from tests.circuits import (CHANNELS, expectation_atol, gradient_atol, random_circuit,
                            random_paulisum)
from tests.stats import bits_to_index, chi2_pvalue

pytestmark = pytest.mark.gpu

c_i64, c_i32, c_u64, vp = ctypes.c_int64, ctypes.c_int32, ctypes.c_uint64, ctypes.c_void_p


def _p(a):
    return a.ctypes.data_as(vp)


def _inputs(seed, nqs, n_ops=2, channels=()):
    rng = np.random.default_rng(seed)
    names = ["a", "b", "c"]
    programs, psums = [], []
    for n in nqs:
        qs = S.GridQubit.rect(1, n)
        c = random_circuit(qs, 5, rng, names, p_control=0.2, channels=list(channels),
                           p_channel=0.3 if channels else 0.0)
        programs.append(S.serialize_circuit(c))
        psums.append([random_paulisum(qs, rng) for _ in range(n_ops)])
    values = rng.uniform(-2, 2, size=(len(nqs), 3)).astype(np.float32)
    return programs, names, values, psums


def _strings(programs, names, psums=None):
    out = [_native.string_array(programs), _native.string_array(names)]
    if psums is not None:
        out.append(_native.string_array([x for row in psums for x in row]))
    return out


def test_max_num_qubits_and_state_with_padding():
    lib = _native.lib()
    programs, names, values, _ = _inputs(1, [3, 7, 5])
    (pp, pl, k1), (npp, npl, k2) = _strings(programs, names)
    lib.tfqg_max_num_qubits.argtypes = [vp, vp, c_i64, vp]
    mq = c_i32()
    assert lib.tfqg_max_num_qubits(pp, pl, 3, ctypes.byref(mq)) == 0
    assert mq.value == 7
    lib.tfqg_simulate_state.argtypes = [vp, vp, c_i64, vp, vp, c_i64, vp, c_i32, vp]
    out = np.zeros((3, 2 ** 7), np.complex64)
    v = np.ascontiguousarray(values)
    assert lib.tfqg_simulate_state(pp, pl, 3, npp, npl, 3, _p(v), 7, _p(out)) == 0
    np.testing.assert_allclose(out, O.simulate_state(programs, names, values), atol=1e-5,
                               rtol=0)
    # a wrong width is refused, not written past
    rc = lib.tfqg_simulate_state(pp, pl, 3, npp, npl, 3, _p(v), 6, _p(out))
    assert rc == 3 and b"max_num_qubits" in lib.tfqg_last_error()


def test_samples_layout_and_distribution():
    lib = _native.lib()
    programs, names, values, _ = _inputs(2, [6, 3])
    (pp, pl, k1), (npp, npl, k2) = _strings(programs, names)
    lib.tfqg_simulate_samples.argtypes = [vp, vp, c_i64, vp, vp, c_i64, vp, c_i32, c_u64,
                                          c_i32, vp]
    shots = 20000
    out = np.zeros((2, shots, 6), np.int8)
    v = np.ascontiguousarray(values)
    assert lib.tfqg_simulate_samples(pp, pl, 2, npp, npl, 3, _p(v), shots, 99, 6, _p(out)) == 0
    assert (out[1, :, :3] == -2).all()
    for r, (n, probs) in enumerate(O.final_probabilities(programs, names, values)):
        counts = np.bincount(bits_to_index(out[r], n), minlength=2 ** n)
        p, _, _ = chi2_pvalue(counts, probs, shots)
        assert p > 1e-3
    assert lib.tfqg_simulate_samples(pp, pl, 2, npp, npl, 3, _p(v), -1, 99, 6, _p(out)) == 3
    # zero samples: an empty output, as the reference op returns
    assert lib.tfqg_simulate_samples(pp, pl, 2, npp, npl, 3, _p(v), 0, 99, 6, _p(out)) == 0


def test_expectation_and_adjoint_gradient():
    lib = _native.lib()
    programs, names, values, psums = _inputs(3, [4, 9, 13])
    (pp, pl, k1), (npp, npl, k2), (spp, spl, k3) = _strings(programs, names, psums)
    v = np.ascontiguousarray(values)
    e = np.zeros((3, 2), np.float32)
    lib.tfqg_simulate_expectation.argtypes = [vp, vp, c_i64, vp, vp, c_i64, vp, vp, vp,
                                              c_i64, vp]
    assert lib.tfqg_simulate_expectation(pp, pl, 3, npp, npl, 3, _p(v), spp, spl, 2,
                                         _p(e)) == 0
    np.testing.assert_allclose(e, O.simulate_expectation(programs, names, values, psums),
                               atol=expectation_atol(psums), rtol=0)
    dg = np.ascontiguousarray(np.random.default_rng(4).normal(size=(3, 2)).astype(np.float32))
    g = np.zeros((3, 3), np.float32)
    lib.tfqg_adj_grad.argtypes = lib.tfqg_simulate_expectation.argtypes[:10] + [vp, vp]
    assert lib.tfqg_adj_grad(pp, pl, 3, npp, npl, 3, _p(v), spp, spl, 2, _p(dg), _p(g)) == 0
    np.testing.assert_allclose(g, O.adj_grad(programs, names, values, psums, dg),
                               atol=gradient_atol(psums, dg), rtol=0)


def test_noisy_and_sampled_expectation():
    lib = _native.lib()
    programs, names, values, psums = _inputs(5, [3, 4], channels=CHANNELS)
    (pp, pl, k1), (npp, npl, k2), (spp, spl, k3) = _strings(programs, names, psums)
    v = np.ascontiguousarray(values)
    R = 20000
    reps = np.full((2, 2), R, np.int32)
    out = np.zeros((2, 2), np.float32)
    args = [vp, vp, c_i64, vp, vp, c_i64, vp, vp, vp, c_i64, vp, c_u64, vp]
    lib.tfqg_noisy_expectation.argtypes = args
    assert lib.tfqg_noisy_expectation(pp, pl, 2, npp, npl, 3, _p(v), spp, spl, 2, _p(reps),
                                      7, _p(out)) == 0
    want = O.noisy_expectation_exact(programs, names, values, psums)
    # std of a bounded observable's trajectory mean <= sum|c| / sqrt(R)
    bound = 5 * expectation_atol(psums, 1.0) / np.sqrt(R)
    np.testing.assert_allclose(out, want, atol=bound, rtol=0)
    programs, names, values, psums = _inputs(6, [3, 5])
    (pp, pl, k1), (npp, npl, k2), (spp, spl, k3) = _strings(programs, names, psums)
    v = np.ascontiguousarray(values)
    lib.tfqg_simulate_sampled_expectation.argtypes = args
    assert lib.tfqg_simulate_sampled_expectation(pp, pl, 2, npp, npl, 3, _p(v), spp, spl, 2,
                                                 _p(reps), 8, _p(out)) == 0
    want = O.simulate_expectation(programs, names, values, psums)
    np.testing.assert_allclose(out, want, atol=bound, rtol=0)


def test_inner_product():
    lib = _native.lib()
    rng = np.random.default_rng(9)
    qs = S.GridQubit.rect(1, 4)
    names = ["a", "b", "c"]
    programs = [S.serialize_circuit(random_circuit(qs, 4, rng, names)) for _ in range(2)]
    others = [[S.serialize_circuit(random_circuit(qs, 4, rng, [])) for _ in range(3)]
              for _ in range(2)]
    values = rng.uniform(-2, 2, size=(2, 3)).astype(np.float32)
    (pp, pl, k1), (npp, npl, k2) = _strings(programs, names)
    opp, opl, k3 = _native.string_array([x for row in others for x in row])
    out = np.zeros((2, 3), np.complex64)
    v = np.ascontiguousarray(values)
    lib.tfqg_inner_product.argtypes = [vp, vp, c_i64, vp, vp, c_i64, vp, vp, vp, c_i64, vp]
    assert lib.tfqg_inner_product(pp, pl, 2, npp, npl, 3, _p(v), opp, opl, 3, _p(out)) == 0
    np.testing.assert_allclose(out, O.inner_product(programs, names, values, others),
                               atol=1e-5, rtol=0)
