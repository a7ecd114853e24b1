"""Parity of the CUDA path (through the C ABI) against the complex128 oracle.

Tolerances: expectations 1e-5 absolute per unit of the observable's
sum_t |c_t| (the reference's own op tests use atol=rtol=1e-5 against cirq,
circuit_execution_ops_test.py:189, on unit-weight observables); gradients
1e-5 per unit of the weighted observable sum_j |g_j| sum_t |c_t|; states
1e-5 (tests/circuits.py expectation_atol, gradient_atol)."""

import numpy as np
import pytest

from quantum_gb300 import ops
from quantum_gb300 import serialize as S
from oracle import tfq_oracle as O
from tests.circuits import (CHANNELS, expectation_atol, gradient_atol, random_circuit,
                            random_paulisum)

pytestmark = pytest.mark.gpu


def _batch(rng, nqs, n_moments, n_symbols=6, n_ops=2, p_control=0.3,
           grid=True):
    names = [f"s{i}" for i in range(n_symbols)]
    programs, psums = [], []
    for n in nqs:
        qs = S.GridQubit.rect(1, n) if grid else S.LineQubit.range(n)
        c = random_circuit(qs, n_moments, rng, names, p_control=p_control)
        programs.append(S.serialize_circuit(c))
        psums.append([random_paulisum(qs, rng) for _ in range(n_ops)])
    values = rng.uniform(-2, 2, size=(len(nqs), n_symbols)).astype(np.float32)
    return programs, names, values, psums


@pytest.mark.parametrize("nqs", [[1, 2, 3], [4, 5, 6], [8, 8], [10, 12],
                                 [13], [14], [15], [16, 9]])
def test_expectation_matches_oracle(nqs):
    rng = np.random.default_rng(sum(nqs) * 7 + len(nqs))
    programs, names, values, psums = _batch(rng, nqs, 6)
    got = ops.tfq_simulate_expectation(programs, names, values, psums)
    want = O.simulate_expectation(programs, names, values, psums)
    np.testing.assert_allclose(got, want, atol=expectation_atol(psums), rtol=0)


@pytest.mark.parametrize("nqs", [[2, 3], [1, 5, 8], [14, 3], [15, 2]])
def test_state_matches_oracle_with_padding(nqs):
    rng = np.random.default_rng(100 + sum(nqs))
    programs, names, values, _ = _batch(rng, nqs, 5, n_ops=0)
    got = ops.tfq_simulate_state(programs, names, values)
    want = O.simulate_state(programs, names, values)
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, atol=1e-5, rtol=0)


def test_expectation_golden_util_qsim():
    """util_qsim_test.cc:119-182: 0.1234 * {ZZ,...,YY} on a fixed state."""
    q = S.LineQubit.range(2)
    prog = S.serialize_circuit(S.Circuit([[S.XPow(q[0], 0.25)],
                                          [S.CNOT(q[0], q[1])],
                                          [S.YPow(q[1], 0.5)]]))
    cases = [("ZZ", 0.0), ("ZX", 0.1234), ("ZY", 0.0), ("XZ", 0.0),
             ("XX", 0.0), ("XY", -0.08725), ("YZ", 0.08725), ("YX", 0.0),
             ("YY", 0.0)]
    psums = [[S.serialize_paulisum([(0.1234, [(q[0], p[0]), (q[1], p[1])])])
              for p, _ in cases]]
    got = ops.tfq_simulate_expectation([prog], [], np.zeros((1, 0)), psums)
    np.testing.assert_allclose(got[0], [v for _, v in cases], atol=1e-5)


def test_expectation_empty_and_identity():
    q = S.GridQubit.rect(1, 2)
    prog = S.serialize_circuit(S.Circuit([[S.H(q[0])], [S.CNOT(q[0], q[1])]]))
    empty = S.serialize_circuit(S.Circuit())
    ps = S.serialize_paulisum([(0.5, []), (2.0, [(q[0], "Z"), (q[1], "Z")])])
    got = ops.tfq_simulate_expectation([prog, empty], [], np.zeros((2, 0)),
                                       [[ps], [ps]])
    np.testing.assert_allclose(got, [[2.5], [-2.0]], atol=1e-6)


@pytest.mark.parametrize("nqs,rule", [([2, 3, 4], 0), ([6, 7], 1),
                                      ([10, 12], 0), ([13], 1), ([14], 0),
                                      ([15, 5], 1)])
def test_adj_grad_matches_oracle(nqs, rule):
    rng = np.random.default_rng(1000 + sum(nqs) + rule)
    programs, names, values, psums = _batch(rng, nqs, 5, n_symbols=5)
    dg = rng.normal(size=(len(nqs), len(psums[0]))).astype(np.float32)
    got = ops.tfq_adj_grad(programs, names, values, psums, dg, grad_rule=rule)
    want = O.adj_grad(programs, names, values, psums, dg,
                      grad_rule="fd" if rule == 0 else "analytic")
    np.testing.assert_allclose(got, want, atol=gradient_atol(psums, dg), rtol=0)


@pytest.mark.parametrize("case", [
    ("GridQubit", [("XP", "alpha"), ("YP", "beta")], None,
     ["alpha", "beta"], [0.123, 0.456], [-1.18392, 0.43281]),
    ("GridQubit", [("XP", "alpha"), ("YP", "beta")], ("gamma", 0.5),
     ["alpha", "beta", "gamma"], [0.123, 0.456, 0.789], [-2.100, -1.7412, -1.5120]),
    ("GridQubit", [("XP", "alpha"), ("YP", "beta")], ("gamma", "gamma"),
     ["alpha", "beta", "gamma"], [0.123, 0.456, 0.789], [-2.3484, -1.7532, -1.64264]),
    ("LineQubit", [("XP", "alpha"), ("YP", "alpha")], (-0.56, "alpha"),
     ["alpha", "beta", "gamma"], [0.123, 0.456, 0.789], [1.2993, 0, 0]),
])
def test_adj_grad_reference_goldens(case):
    """tfq_adj_grad_op_test.py:265-397 (atol 1e-3 there)."""
    qtype, singles, fsim, names, vals, want = case
    q = S.GridQubit.rect(1, 2) if qtype == "GridQubit" else S.LineQubit.range(2)
    moments = [[S.XPow(q[0], S.Symbol(singles[0][1]))],
               [S.YPow(q[1], S.Symbol(singles[1][1]))],
               [S.CNOT(q[0], q[1])]]
    if fsim is not None:
        th, ph = fsim
        th = S.Symbol(th) if isinstance(th, str) else th
        ph = S.Symbol(ph) if isinstance(ph, str) else ph
        moments.append([S.FSim(q[0], q[1], th, ph)])
    prog = S.serialize_circuit(S.Circuit(moments))
    psums = [[S.serialize_paulisum([(1.0, [(q[0], "Z")])]),
              S.serialize_paulisum([(1.0, [(q[1], "X")])])]]
    got = ops.tfq_adj_grad([prog], names, np.array([vals], np.float32), psums,
                           np.ones((1, 2), np.float32))
    np.testing.assert_allclose(got[0], want, atol=1e-3)


def test_adj_grad_empty_rows_and_no_ops():
    q = S.GridQubit.rect(1, 2)
    prog = S.serialize_circuit(S.Circuit([[S.XPow(q[0], S.Symbol("a"))]]))
    empty = S.serialize_circuit(S.Circuit())
    ps = S.serialize_paulisum([(1.0, [(q[0], "Z")])])
    got = ops.tfq_adj_grad([prog, empty], ["a"], np.full((2, 1), 0.3, np.float32),
                           [[ps], [ps]], np.ones((2, 1), np.float32))
    assert got[1, 0] == 0.0
    want = O.adj_grad([prog, empty], ["a"], np.full((2, 1), 0.3), [[ps], [ps]],
                      np.ones((2, 1)))
    np.testing.assert_allclose(got, want, atol=1e-5)


def test_samples_bit_layout_and_padding():
    """tfq_simulate_ops_test.py:467-492: X on every qubit -> all ones in the
    trailing n columns, -2 in the leading max_n - n."""
    for all_n in ([2, 3], [1, 5, 8]):
        circuits = [S.serialize_circuit(S.Circuit(
            [[S.X(q) for q in S.GridQubit.rect(1, n)]])) for n in all_n]
        res = ops.tfq_simulate_samples(circuits, [], np.zeros((len(all_n), 0)),
                                       [10])
        m = max(all_n)
        for i, n in enumerate(all_n):
            exp = np.zeros((10, m))
            exp[:, m - n:] = 1
            exp[:, :m - n] = -2
            np.testing.assert_array_equal(res[i], exp)


@pytest.mark.parametrize("n", [3, 6, 15])
def test_samples_distribution_chi2(n):
    """Sampled bitstrings follow |psi|^2 (chi-squared, p > 1e-3)."""
    from scipy import stats
    rng = np.random.default_rng(77 + n)
    qs = S.GridQubit.rect(1, n)
    c = random_circuit(qs, 4, rng, [], p_control=0.2)
    prog = S.serialize_circuit(c)
    shots = 40000
    res = ops.tfq_simulate_samples([prog], [], np.zeros((1, 0)), [shots], seed=1234)
    bits = res[0].astype(np.int64)
    idx = np.zeros(shots, dtype=np.int64)
    for col in range(n):  # column col holds qubit col (big-endian index)
        idx = (idx << 1) | bits[:, col]
    (_, probs), = O.final_probabilities([prog], [], np.zeros((1, 0)))
    counts = np.bincount(idx, minlength=2 ** n)
    exp = probs * shots
    # merge bins with fewer than 5 expected counts
    order = np.argsort(exp)
    ce, cc, acc_e, acc_c = [], [], 0.0, 0
    for k in order:
        acc_e += exp[k]
        acc_c += counts[k]
        if acc_e >= 5:
            ce.append(acc_e)
            cc.append(acc_c)
            acc_e, acc_c = 0.0, 0
    if acc_e > 0 and ce:
        ce[-1] += acc_e
        cc[-1] += acc_c
    chi2 = float(np.sum((np.array(cc) - np.array(ce)) ** 2 / np.array(ce)))
    p = stats.chi2.sf(chi2, max(len(ce) - 1, 1))
    assert p > 1e-3, (chi2, len(ce), p)


@pytest.mark.parametrize("n,channels", [(3, CHANNELS), (5, ["DP", "AD", "PD"]),
                                        (4, ["GAD", "RST", "BF", "PF", "ADP"])])
def test_noisy_expectation_vs_density_matrix(n, channels):
    """Trajectory mean vs exact density matrix (the reference checks 5e-2 at
    10000 trajectories, noise/noisy_expectation_op_test.py:224-274); here the
    bound is 5 standard errors."""
    rng = np.random.default_rng(500 + n)
    qs = S.GridQubit.rect(1, n)
    names = ["a", "b"]
    progs, psums = [], []
    for _ in range(2):
        c = random_circuit(qs, 5, rng, names, p_control=0.2,
                           channels=list(channels), p_channel=0.4)
        progs.append(S.serialize_circuit(c))
        psums.append([S.serialize_paulisum([(1.0, [(q, "Z")]) for q in qs]),
                      random_paulisum(qs, rng)])
    vals = rng.uniform(-1, 1, size=(2, 2)).astype(np.float32)
    R = 20000
    got = ops.noisy_expectation(progs, names, vals, psums,
                                np.full((2, 2), R, np.int32), seed=7)
    want = O.noisy_expectation_exact(progs, names, vals, psums)
    # std of a bounded observable's trajectory mean <= sum|c| / sqrt(R)
    bound = 5 * n / np.sqrt(R) + 1e-4
    np.testing.assert_allclose(got, want, atol=bound, rtol=0)


def test_noisy_without_noise_matches_expectation():
    rng = np.random.default_rng(9)
    programs, names, values, psums = _batch(rng, [4, 6], 5)
    got = ops.noisy_expectation(programs, names, values, psums,
                                np.full((2, 2), 3, np.int32), seed=1)
    want = O.simulate_expectation(programs, names, values, psums)
    np.testing.assert_allclose(got, want, atol=1e-4)


def test_torch_autograd_cuda():
    import torch
    rng = np.random.default_rng(21)
    programs, names, values, psums = _batch(rng, [5, 6, 7], 5)
    from quantum_gb300.torch_ops import Expectation
    layer = Expectation(programs, names, psums)
    v = torch.tensor(values, device="cuda", requires_grad=True)
    e = layer(v)
    w = torch.tensor(rng.normal(size=e.shape).astype(np.float32), device="cuda")
    (e * w).sum().backward()
    want_e = O.simulate_expectation(programs, names, values, psums)
    want_g = O.adj_grad(programs, names, values, psums, w.cpu().numpy())
    np.testing.assert_allclose(e.detach().cpu().numpy(), want_e, atol=1e-4)
    np.testing.assert_allclose(v.grad.cpu().numpy(), want_g, atol=1e-4)


@pytest.mark.parametrize("nqs", [[3, 5], [8, 12], [16]])
def test_sampled_expectation_matches_exact_within_sampling_error(nqs):
    """tfq_simulate_sampled_expectation: the estimate of each op is a sum over
    terms of coef * mean parity; its standard deviation is
    sqrt(sum_t coef_t^2 (1 - <P_t>^2) / N).  Checked at 5 standard deviations
    against the oracle's exact expectation."""
    rng = np.random.default_rng(300 + sum(nqs))
    programs, names, values, psums = _batch(rng, nqs, 5)
    N = 20000
    ns = np.full((len(nqs), 2), N, np.int32)
    got = ops.tfq_simulate_sampled_expectation(programs, names, values, psums, ns, seed=17)
    want = O.simulate_expectation(programs, names, values, psums)
    coefs = []
    for row in psums:
        coefs.append([sum(c * c for c, _ in _terms(p)) for p in row])
    bound = 5 * np.sqrt(np.asarray(coefs) / N) + 1e-5
    assert np.all(np.abs(got - want) <= bound), (got, want, bound)
    # the same seed reproduces the draws
    again = ops.tfq_simulate_sampled_expectation(programs, names, values, psums, ns, seed=17)
    np.testing.assert_array_equal(got, again)


def _terms(paulisum_bytes):
    """(coefficient, paulis) of the non-identity terms of a serialized sum."""
    return [(float(t["re"]), t["paulis"]) for t in O.decode_paulisum(paulisum_bytes)
            if t["paulis"]]


def test_sampled_expectation_empty_program_and_identity():
    q = S.GridQubit.rect(1, 2)
    prog = S.serialize_circuit(S.Circuit([[S.X(q[0]), S.I(q[1])]]))
    empty = S.serialize_circuit(S.Circuit([]))
    ps = S.serialize_paulisum([(0.5, []), (2.0, [(q[0], "Z")])])
    got = ops.tfq_simulate_sampled_expectation([prog, empty], [], np.zeros((2, 0)),
                                               [[ps], [ps]], np.full((2, 1), 100, np.int32))
    # X|0> = |1>: Z = -1 exactly, so every parity is -1
    np.testing.assert_allclose(got, [[0.5 - 2.0], [-2.0]], atol=1e-6)


def test_text_format_inputs_give_identical_results():
    """Programs and pauli sums given in protobuf text format (the reference's
    TextFormat fallback, parse_context.cc:155-170) run exactly like binary."""
    from tests import textfmt
    rng = np.random.default_rng(77)
    programs, names, values, psums = _batch(rng, [4, 7, 12], 5)
    tp = [textfmt.to_text(p).encode() for p in programs]
    tps = [[textfmt.to_text(x, "PauliSum").encode() for x in row] for row in psums]
    np.testing.assert_array_equal(ops.tfq_simulate_expectation(tp, names, values, tps),
                                  ops.tfq_simulate_expectation(programs, names, values, psums))


@pytest.mark.parametrize("n", [2, 15])
def test_identity_only_program_is_not_empty(n):
    """A program of identity gates has a non-empty fused circuit in the
    reference, so its expectation is taken on |0...0> (not the -2 of an
    empty program), resident (2 qubits) or streamed (15 qubits)."""
    q = S.GridQubit.rect(1, n)
    prog = S.serialize_circuit(S.Circuit([[S.I(x) for x in q]]))
    ps = S.serialize_paulisum([(0.5, [(q[0], "Z")]), (0.25, [])])
    got = ops.tfq_simulate_expectation([prog], [], np.zeros((1, 0)), [[ps]])
    np.testing.assert_allclose(got, [[0.75]], atol=1e-6)
    st = ops.tfq_simulate_state([prog], [], np.zeros((1, 0)))
    assert st[0, 0] == 1 and np.all(st[0, 1:] == 0)


def test_inner_product_docstring_example():
    """math_ops/inner_product_op.py:72-130 (the reference's documented output)."""
    import json, os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                    "reference_goldens.json")))["inner_product"]
    q = S.GridQubit.rect(1, 2)
    a, b = S.Symbol("alpha"), S.Symbol("beta")
    ref = [S.serialize_circuit(S.Circuit([[S.HPow(x, a) for x in q]])),
           S.serialize_circuit(S.Circuit([[S.XPow(q[0], a), S.YPow(q[1], b)]]))]
    oth = [S.serialize_circuit(S.Circuit([[S.X(x) for x in q]])),
           S.serialize_circuit(S.Circuit([[S.YPow(x, 0.125) for x in q]])),
           S.serialize_circuit(S.Circuit([[S.XPow(x, 0.5) for x in q]]))]
    got = ops.tfq_inner_product(ref, ["alpha", "beta"], np.array(g["values"], np.float32),
                                [oth, oth])
    want = np.array([[complex(*z) for z in r] for r in g["out"]])
    np.testing.assert_allclose(got, want, atol=g["tolerance"])


@pytest.mark.parametrize("n,others", [(3, 2), (9, 3), (14, 1), (17, 2)])
def test_inner_product_matches_oracle(n, others):
    rng = np.random.default_rng(900 + n)
    qs = S.GridQubit.rect(1, n)
    names = ["a", "b"]
    refs, oth = [], []
    for _ in range(2):
        refs.append(S.serialize_circuit(random_circuit(qs, 5, rng, names, p_control=0.3)))
        oth.append([S.serialize_circuit(random_circuit(qs, 4, rng, (), p_control=0.3))
                    for _ in range(others)])
    values = rng.uniform(-2, 2, size=(2, 2)).astype(np.float32)
    got = ops.tfq_inner_product(refs, names, values, oth)
    want = O.inner_product(refs, names, values, oth)
    assert got.dtype == np.complex64 and got.shape == want.shape
    np.testing.assert_allclose(got, want, atol=1e-5, rtol=0)


@pytest.mark.parametrize("n,others", [(3, 2), (8, 3), (13, 1), (15, 2)])
def test_inner_product_grad_matches_oracle(n, others):
    """TfqInnerProductGrad (math_ops/tfq_inner_product_grad.cc): complex
    sum_j g_ij <dU psi_i | phi_ij> per symbol with the reference's FD
    gradient gates; resident (3, 8, 13 qubits) and streamed (15)."""
    rng = np.random.default_rng(950 + n)
    qs = S.GridQubit.rect(1, n)
    names = ["a", "b", "c"]
    refs, oth = [], []
    for _ in range(2):
        refs.append(S.serialize_circuit(random_circuit(qs, 4, rng, names, p_control=0.3)))
        oth.append([S.serialize_circuit(random_circuit(qs, 3, rng, (), p_control=0.3))
                    for _ in range(others)])
    refs.append(S.serialize_circuit(S.Circuit()))  # empty reference: zero row
    oth.append(list(oth[0]))
    values = rng.uniform(-2, 2, size=(3, 3)).astype(np.float32)
    dg = rng.normal(size=(3, others)).astype(np.float32)
    b = ops.InnerProductBatch(refs, names, oth, with_grads=True)
    got = b.inner_product_grad(values, dg)
    want = O.inner_product_grad(refs, names, values, oth, dg)
    scale = max(1.0, float(np.abs(want).max()))
    np.testing.assert_allclose(got, want, atol=2e-5 * scale, rtol=0)
    assert np.all(got[2] == 0)
    np.testing.assert_allclose(
        ops.inner_product_grad(refs, names, values, oth, dg), np.conj(want),
        atol=2e-5 * scale, rtol=0)


def test_noisy_samples_distribution_and_layout():
    """tfq.noise.samples (noise/tfq_noisy_samples.cc): one measurement per
    trajectory; the sample histogram against the exact density matrix's
    diagonal (chi-squared, p > 1e-3), the samples op's bit layout and -2
    padding, and an empty program padded throughout."""
    rng = np.random.default_rng(41)
    q3 = S.GridQubit.rect(1, 3)
    c = random_circuit(q3, 5, rng, ["a"], p_control=0.2, channels=list(CHANNELS),
                       p_channel=0.4)
    prog3 = S.serialize_circuit(c)
    q2 = S.GridQubit.rect(1, 2)
    prog2 = S.serialize_circuit(S.Circuit([[S.X(q2[0]), S.I(q2[1])],
                                           [S.bit_flip(q2[1], 0.25)]]))
    empty = S.serialize_circuit(S.Circuit())
    vals = np.array([[0.4], [0.0], [0.0]], np.float32)
    shots = 20000
    res = ops.noisy_samples([prog3, prog2, empty], ["a"], vals, [shots], seed=3)
    assert res.shape == (3, shots, 3)
    assert (res[2] == -2).all()
    assert (res[1, :, 0] == -2).all() and (res[1, :, 1] == 1).all()
    flips = res[1, :, 2].mean()
    assert abs(flips - 0.25) < 5 * np.sqrt(0.25 * 0.75 / shots)
    from scipy import stats
    (n, probs), *_ = O.noisy_probabilities([prog3], ["a"], vals[:1])
    idx = (res[0].astype(np.int64)[:, ::-1] << np.arange(3)).sum(axis=1)
    counts = np.bincount(idx, minlength=8)
    exp = probs * shots
    keep = exp >= 5
    cc = list(counts[keep]) + [counts[~keep].sum()]
    ce = list(exp[keep]) + [exp[~keep].sum()]
    if ce[-1] < 5:
        cc[-2] += cc.pop()
        ce[-2] += ce.pop()
    p = stats.chisquare(cc, np.asarray(ce) * sum(cc) / sum(ce)).pvalue
    assert p > 1e-3, (counts, probs, p)


@pytest.mark.parametrize("n,channels", [(3, CHANNELS), (5, ["DP", "AD", "BF"])])
def test_noisy_sampled_expectation_vs_density_matrix(n, channels):
    """tfq.noise.sampled_expectation: each trajectory measures every term once;
    the mean of R trajectories is within 5 standard errors (sum|c| / sqrt(R))
    of the exact density-matrix expectation; empty programs give -2."""
    rng = np.random.default_rng(610 + n)
    qs = S.GridQubit.rect(1, n)
    names = ["a", "b"]
    progs, psums = [], []
    for _ in range(2):
        c = random_circuit(qs, 5, rng, names, p_control=0.2, channels=list(channels),
                           p_channel=0.4)
        progs.append(S.serialize_circuit(c))
        psums.append([S.serialize_paulisum([(1.0, [(q, "Z")]) for q in qs]),
                      random_paulisum(qs, rng)])
    progs.append(S.serialize_circuit(S.Circuit()))
    psums.append(psums[0])
    vals = rng.uniform(-1, 1, size=(3, 2)).astype(np.float32)
    R = 20000
    got = ops.noisy_sampled_expectation(progs, names, vals, psums,
                                        np.full((3, 2), R, np.int32), seed=9)
    want = O.noisy_expectation_exact(progs[:2], names, vals[:2], psums[:2])
    absc = [[sum(abs(float(t["re"])) for t in O.decode_paulisum(p) if t["paulis"])
             for p in row] for row in psums[:2]]
    bound = 5 * np.asarray(absc) / np.sqrt(R) + 1e-4
    assert np.all(np.abs(got[:2] - want) <= bound), (got, want, bound)
    np.testing.assert_array_equal(got[2], [-2.0, -2.0])


@pytest.mark.parametrize("case", ["layers", "grid", "uneven", "random"])
def test_fused_forward_plans_match_unfused_and_oracle(case):
    """Forward plans run fused gates (one-qubit chains folded into two-qubit
    gates); states and expectations must match the unfused plan and the
    oracle, resident (<= 14 qubits) and streamed (15, 16 qubits) alike."""
    from quantum_gb300 import _native, workloads
    rng = np.random.default_rng(17)
    if case == "layers":
        w = workloads.expectation_layers(batch=4, n=15, layers=3, seed=2)
        programs, names, values = w["programs"], w["symbol_names"], w["symbol_values"]
        psums = w["pauli_sums"]
    elif case == "grid":
        w = workloads.grid_fsim(rows=4, cols=4, depth=10, seed=3)
        programs, names, values = w["programs"], [], np.zeros((1, 0), np.float32)
        psums = w["pauli_sums"]
    elif case == "uneven":
        w = workloads.uneven_batch(batch=24, n_min=4, n_max=16, d_min=4, d_max=12, seed=5)
        programs, names, values = w["programs"], [], w["symbol_values"]
        psums = w["pauli_sums"]
    else:
        programs, names, values, psums = _batch(rng, [3, 7, 12, 15], 10, n_ops=1)
    want_e = O.simulate_expectation(programs, names, values, psums)
    want_s = O.simulate_state(programs, names, values)
    results = {}
    for fuse in (True, False):
        prev = _native.set_gate_fusion(fuse)
        try:
            b = ops.Batch(programs, names, psums, kind=ops.KIND_FORWARD)
        finally:
            _native.set_gate_fusion(prev)
        results[fuse] = (b.expectation(values), b.state(values))
        b.close()
    for fuse, (e, s) in results.items():
        np.testing.assert_allclose(e, want_e, atol=expectation_atol(psums), rtol=0)
        np.testing.assert_allclose(s, want_s, atol=1e-5, rtol=0)


@pytest.mark.parametrize("n,channels", [(16, ["AD", "GAD", "RST", "PD", "DP"]),
                                        (15, ["AD", "PD", "BF", "GAD"])])
def test_streamed_non_unitary_channels_vs_density_matrix(n, channels):
    """Channels whose branch probabilities are state norms (amplitude and
    phase damping, reset, GAD) on streamed states (> 14 qubits): a 6-qubit
    noisy circuit on qubits spread over high, middle and low index bits,
    embedded in n qubits whose other qubits only get rotations. Observables
    on the active qubits must match the 6-qubit exact density matrix."""
    rng = np.random.default_rng(900 + n)
    qs = S.GridQubit.rect(1, n)
    active = [qs[i] for i in (0, 1, n // 2 - 1, n // 2 + 2, n - 2, n - 1)]
    idle = [q for q in qs if q not in active]
    names = ["a", "b"]
    c = random_circuit(active, 6, rng, names, p_control=0.2,
                       channels=list(channels), p_channel=0.45)
    full = S.Circuit([[S.rx(q, float(rng.uniform(0, 3))) for q in idle]] + c.moments
                     + [[S.ry(q, float(rng.uniform(0, 3))) for q in idle]])
    psums = [[S.serialize_paulisum([(1.0, [(q, "Z")]) for q in active]),
              random_paulisum(active, rng)]]
    vals = rng.uniform(-1, 1, size=(1, 2)).astype(np.float32)
    R = 12000
    got = ops.noisy_expectation([S.serialize_circuit(full)], names, vals, psums,
                                np.full((1, 2), R, np.int32), seed=11)
    want = O.noisy_expectation_exact([S.serialize_circuit(c)], names, vals, psums)
    bound = 5 * len(active) / np.sqrt(R) + 1e-4
    np.testing.assert_allclose(got, want, atol=bound, rtol=0)
