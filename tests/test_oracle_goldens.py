"""The oracle pinned against the reference's own known-answer tests
(tests/golden/reference_goldens.json, literals from the reference test files)."""

import json
import os

import numpy as np
import pytest

from oracle import tfq_oracle as O
from quantum_gb300 import serialize as S

G = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                "reference_goldens.json")))


def test_util_qsim_two_term_expectations():
    g = G["util_qsim_two_term"]
    q = S.LineQubit.range(2)
    prog = S.serialize_circuit(S.Circuit([[S.XPow(q[0], 0.25)],
                                          [S.CNOT(q[0], q[1])],
                                          [S.YPow(q[1], 0.5)]]))
    names = list(g["values"])
    psums = [[S.serialize_paulisum([(g["coefficient"], [(q[0], p[0]), (q[1], p[1])])])
              for p in names]]
    got = O.simulate_expectation([prog], [], np.zeros((1, 0)), psums)[0]
    np.testing.assert_allclose(got, [g["values"][p] for p in names],
                               atol=g["tolerance"])


def test_identity_term():
    g = G["util_qsim_identity"]
    q = S.LineQubit.range(2)
    prog = S.serialize_circuit(S.Circuit([[S.I(q[0]), S.I(q[1])]]))
    ps = [[S.serialize_paulisum([(g["coefficient"], [])])]]
    got = O.simulate_expectation([prog], [], np.zeros((1, 0)), ps)[0, 0]
    assert abs(got - g["value"]) < g["tolerance"]


def _golden_circuit(case):
    q = S.GridQubit.rect(1, 2) if case["qubits"] == "grid" else S.LineQubit.range(2)
    moments = []
    for op in case["circuit"]:
        gid = op[0]
        if gid in ("XP", "YP"):
            ctor = S.XPow if gid == "XP" else S.YPow
            moments.append([ctor(q[op[1]], S.Symbol(op[2]))])
        elif gid == "CNP":
            moments.append([S.CNOT(q[op[1]], q[op[2]])])
        else:
            th, ph = op[3], op[4]
            th = S.Symbol(th) if isinstance(th, str) else th
            ph = S.Symbol(ph) if isinstance(ph, str) else ph
            moments.append([S.FSim(q[op[1]], q[op[2]], th, ph)])
    psums = [[S.serialize_paulisum([(1.0, [(q[0], "Z")])]),
              S.serialize_paulisum([(1.0, [(q[1], "X")])])]]
    return S.serialize_circuit(S.Circuit(moments)), psums


@pytest.mark.parametrize("case", G["adj_grad"]["cases"], ids=lambda c: c["name"])
def test_adj_grad_goldens(case):
    prog, psums = _golden_circuit(case)
    got = O.adj_grad([prog], case["symbols"], np.array([case["values"]]), psums,
                     np.ones((1, 2)))
    np.testing.assert_allclose(got[0], case["grads"], atol=G["adj_grad"]["tolerance"])


@pytest.mark.parametrize("case", G["adj_grad"]["cases"], ids=lambda c: c["name"])
def test_adj_grad_exact_rule_close_to_fd(case):
    """The exact derivative differs from the reference's FD rule by O(eps^2)."""
    prog, psums = _golden_circuit(case)
    fd = O.adj_grad([prog], case["symbols"], np.array([case["values"]]), psums,
                    np.ones((1, 2)))
    ex = O.adj_grad([prog], case["symbols"], np.array([case["values"]]), psums,
                    np.ones((1, 2)), grad_rule="analytic")
    np.testing.assert_allclose(fd, ex, atol=5e-4)


def _op(gid, args):
    return {"gate": gid, "qubits": ["0", "1"][:1 if gid in ("YP", "PXP") else 2],
            "args": {k: {"float": np.float32(v), "symbol": "", "string": ""}
                     for k, v in args.items()}}


@pytest.mark.parametrize("case", G["gradient_gates"]["cases"],
                         ids=lambda c: c["gate"] + "-" + c["param"])
def test_gradient_gate_matrices(case):
    """adj_util_test.cc:355-561: the FD gradient gate of one parameter."""
    op = _op(case["gate"], case["args"])
    op["args"][case["param"]]["symbol"] = "s"
    op["args"]["control_qubits"] = {"float": 0, "symbol": "", "string": ""}
    op["args"]["control_values"] = {"float": 0, "symbol": "", "string": ""}
    index = {"0": 0, "1": 1}
    g = O.build_gate(op, index, {"s": np.float32(case["args"][case["param"]])})
    (_, dm), = g.grads
    want = np.array(case["matrix"]).reshape(-1, 2)
    want = want[:, 0] + 1j * want[:, 1]
    np.testing.assert_allclose(dm.reshape(-1), want, atol=case["tolerance"])


def test_sample_layout_padding():
    """tfq_simulate_samples_op.cc:226-243: bit k -> column maxn-k-1."""
    out = O.sample_bits_layout([0b101, 0b011], 3, 5)
    np.testing.assert_array_equal(out, [[-2, -2, 1, 0, 1], [-2, -2, 0, 1, 1]])


def test_state_padding():
    for all_n in G["padding"]["cases"]:
        progs = [S.serialize_circuit(S.Circuit([[S.H(q) for q in S.GridQubit.rect(1, n)]]))
                 for n in all_n]
        st = O.simulate_state(progs, [], np.zeros((len(all_n), 0)))
        m = max(all_n)
        for i, n in enumerate(all_n):
            np.testing.assert_allclose(st[i, :2 ** n], 2 ** (-n / 2))
            assert np.all(st[i, 2 ** n:] == G["padding"]["state_pad"])
        assert st.shape == (len(all_n), 2 ** m)


def test_density_matrix_matches_statevector_without_noise():
    rng = np.random.default_rng(3)
    from tests.circuits import random_circuit, random_paulisum
    qs = S.GridQubit.rect(1, 3)
    prog = S.serialize_circuit(random_circuit(qs, 4, rng, ["a"]))
    ps = [[random_paulisum(qs, rng)]]
    v = np.array([[0.4]], np.float32)
    a = O.simulate_expectation([prog], ["a"], v, ps)
    b = O.noisy_expectation_exact([prog], ["a"], v, ps)
    np.testing.assert_allclose(a, b, atol=1e-10)


def test_oracle_inner_product_docstring_example():
    """math_ops/inner_product_op.py:72-130: the documented example's output."""
    from quantum_gb300 import serialize as S
    g = G["inner_product"]
    q = S.GridQubit.rect(1, 2)
    a, b = S.Symbol("alpha"), S.Symbol("beta")
    ref = [S.serialize_circuit(S.Circuit([[S.HPow(x, a) for x in q]])),
           S.serialize_circuit(S.Circuit([[S.XPow(q[0], a), S.YPow(q[1], b)]]))]
    oth = [S.serialize_circuit(S.Circuit([[S.X(x) for x in q]])),
           S.serialize_circuit(S.Circuit([[S.YPow(x, 0.125) for x in q]])),
           S.serialize_circuit(S.Circuit([[S.XPow(x, 0.5) for x in q]]))]
    got = O.inner_product(ref, ["alpha", "beta"], np.array(g["values"], np.float32), [oth, oth])
    want = np.array([[complex(*z) for z in r] for r in g["out"]])
    np.testing.assert_allclose(got, want, atol=g["tolerance"])
