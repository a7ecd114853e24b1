"""Writes reference_goldens.json: the reference's own known-answer values for
the state-vector path, with the file:line each comes from.

The reference cannot run in this environment (it needs TensorFlow, cirq and
the qsim external), so its test files are read as text: every value below is
a literal from the cited test.  When a checkout of the reference is named
by TFQ_REFERENCE_DIR, the script checks that each literal still appears in
its cited file.

    TFQ_REFERENCE_DIR=<reference checkout> python tests/golden/make_goldens.py
"""

import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("TFQ_REFERENCE_DIR", "")

GOLDENS = {
    # util_qsim_test.cc:119-182: state prepared by XPow(0.25) on qubit 0,
    # CNOT(0 -> 1), YPow(0.5) on qubit 1 (cirq order; the test builds it
    # with qsim indices 1/0); term 0.1234 * P0 P1; tolerance 1e-5.
    "util_qsim_two_term": {
        "source": "tensorflow_quantum/core/src/util_qsim_test.cc:119-182",
        "coefficient": 0.1234,
        "tolerance": 1e-5,
        "values": {"ZZ": 0.0, "ZX": 0.1234, "ZY": 0.0, "XZ": 0.0, "XX": 0.0,
                   "XY": -0.08725, "YZ": 0.08725, "YX": 0.0, "YY": 0.0},
        "literals": ["0.08725", "0.1234"],
    },
    # util_qsim_test.cc:211-234: identity term contributes its coefficient.
    "util_qsim_identity": {
        "source": "tensorflow_quantum/core/src/util_qsim_test.cc:211-234",
        "coefficient": 0.1234,
        "value": 0.1234,
        "tolerance": 1e-5,
        "literals": ["0.1234"],
    },
    # tfq_adj_grad_op_test.py:265-397, obs [Z(q0), X(q1)], prev_grad = 1.
    "adj_grad": {
        "source": "tensorflow_quantum/core/ops/tfq_adj_grad_op_test.py:265-397",
        "tolerance": 1e-3,
        "cases": [
            {"name": "simple", "qubits": "grid",
             "circuit": [["XP", 0, "alpha"], ["YP", 1, "beta"], ["CNP", 0, 1]],
             "symbols": ["alpha", "beta"], "values": [0.123, 0.456],
             "grads": [-1.18392, 0.43281]},
            {"name": "fsim", "qubits": "grid",
             "circuit": [["XP", 0, "alpha"], ["YP", 1, "beta"], ["CNP", 0, 1],
                         ["FSIM", 0, 1, "gamma", 0.5]],
             "symbols": ["alpha", "beta", "gamma"],
             "values": [0.123, 0.456, 0.789],
             "grads": [-2.100, -1.7412, -1.5120]},
            {"name": "shared", "qubits": "grid",
             "circuit": [["XP", 0, "alpha"], ["YP", 1, "beta"], ["CNP", 0, 1],
                         ["FSIM", 0, 1, "gamma", "gamma"]],
             "symbols": ["alpha", "beta", "gamma"],
             "values": [0.123, 0.456, 0.789],
             "grads": [-2.3484, -1.7532, -1.64264]},
            {"name": "single", "qubits": "line",
             "circuit": [["XP", 0, "alpha"], ["YP", 1, "alpha"], ["CNP", 0, 1],
                         ["FSIM", 0, 1, -0.56, "alpha"]],
             "symbols": ["alpha", "beta", "gamma"],
             "values": [0.123, 0.456, 0.789],
             "grads": [1.2993, 0.0, 0.0]},
        ],
        "literals": ["-1.18392, 0.43281", "-2.100, -1.7412, -1.5120",
                     "-2.3484, -1.7532, -1.64264", "1.2993, 0, 0"],
    },
    # adj_util_test.cc:355-561: gradient-gate matrices (row-major re, im),
    # computed in the test comments by cirq with eps = 1e-4 (1e-3 for the
    # PhasedISwap exponent); tolerances 1e-4 (1e-3 for PhasedISwap phase).
    "gradient_gates": {
        "source": "tensorflow_quantum/core/src/adj_util_test.cc:355-561",
        "cases": [
            {"gate": "YP", "param": "exponent", "args": {"exponent": 0.125,
             "exponent_scalar": 1.0, "global_shift": 0.0}, "tolerance": 1e-4,
             "matrix": [-0.60111, 1.45122, -1.45122, -0.60111,
                        1.45122, 0.60111, -0.60111, 1.45122]},
            {"gate": "XXP", "param": "exponent", "args": {"exponent": 0.001,
             "exponent_scalar": 1.0, "global_shift": 0.0}, "tolerance": 1e-4,
             "matrix": [-0.004934, 1.57078, 0.0, 0.0, 0.0, 0.0, 0.004934,
                        -1.57078, 0.0, 0.0, -0.004934, 1.57078, 0.004934,
                        -1.57078, 0.0, 0.0, 0.0, 0.0, 0.004934, -1.57078,
                        -0.004934, 1.57078, 0.0, 0.0, 0.004934, -1.57078,
                        0.0, 0.0, 0.0, 0.0, -0.004934, 1.57078]},
            {"gate": "PXP", "param": "phase_exponent",
             "args": {"phase_exponent": 10.123, "phase_exponent_scalar": 1.0,
                      "exponent": 1.0, "exponent_scalar": 1.0,
                      "global_shift": 0.0}, "tolerance": 1e-4,
             "matrix": [0.0, 0.0, -1.18397, -2.9099, -1.18397, 2.9099, 0.0, 0.0]},
            {"gate": "PXP", "param": "exponent",
             "args": {"phase_exponent": 10.123, "phase_exponent_scalar": 1.0,
                      "exponent": 0.789, "exponent_scalar": 1.0,
                      "global_shift": 0.0}, "tolerance": 1e-4,
             "matrix": [-0.96664, -1.23814, 1.36199, 0.78254, 0.42875,
                        1.51114, -0.96664, -1.23814]},
            {"gate": "FSIM", "param": "theta",
             "args": {"theta": 0.5, "theta_scalar": 1.0, "phi": 1.2,
                      "phi_scalar": 1.0}, "tolerance": 1e-4,
             "matrix": [0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
                        -0.47942, 0.0, 0.0, -0.87758, 0.0, 0.0, 0.0, 0.0, 0.0,
                        -0.87758, -0.47942, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
                        0.0, 0.0, 0.0, 0.0]},
            {"gate": "FSIM", "param": "phi",
             "args": {"theta": 0.5, "theta_scalar": 1.0, "phi": 1.2,
                      "phi_scalar": 1.0}, "tolerance": 1e-4,
             "matrix": [0.0] * 30 + [-0.932039, -0.362357]},
            {"gate": "PISP", "param": "phase_exponent",
             "args": {"phase_exponent": 8.9, "phase_exponent_scalar": 1.0,
                      "exponent": -3.2, "exponent_scalar": 1.0},
             "tolerance": 1e-3,
             "matrix": [0.0] * 12 + [-4.83441, 3.51238] + [0.0] * 4 +
                       [4.83441, 3.51238] + [0.0] * 12},
            {"gate": "PISP", "param": "exponent",
             "args": {"phase_exponent": 8.9, "phase_exponent_scalar": 1.0,
                      "exponent": -3.2, "exponent_scalar": 1.0},
             "tolerance": 1e-4,
             "matrix": [0.0] * 10 + [-1.49391, 0.0, 0.285312, 0.392698] +
                       [0.0] * 4 + [-0.285312, 0.392698, -1.49391, 0.0] +
                       [0.0] * 10},
        ],
        "literals": ["-0.60111", "-0.004934", "-1.18397", "-0.96664",
                     "-0.47942", "-0.932039", "-4.83441", "-1.49391"],
    },
    # tfq_simulate_ops_test.py:311-346 and :467-492: padding conventions.
    "padding": {
        "source": "tensorflow_quantum/core/ops/tfq_simulate_ops_test.py:311-346,467-492",
        "state_pad": -2.0,
        "sample_pad": -2,
        "cases": [[2, 3], [1, 5, 8]],
        "literals": ["'all_n_qubits': [2, 3]", "'all_n_qubits': [1, 5, 8]"],
    },
    # math_ops/inner_product_op.py:72-130 (docstring example): reference
    # circuits (H**alpha on each qubit) and (X(q0)**alpha, Y(q1)**beta) with
    # values [[0, 1], [2, 3]], paired with X on each qubit, Y**0.125 on each
    # and X**0.5 on each.
    "inner_product": {
        "source": "tensorflow_quantum/core/ops/math_ops/inner_product_op.py:72-130",
        "tolerance": 1e-5,
        "values": [[0, 1], [2, 3]],
        "out": [[[0.0, 0.0], [8.8871640e-01, 0.3681184], [0.0, 0.5]],
                [[0.0, 0.0], [7.3223300e-02, -0.17677669], [0.0, -0.5]]],
        "literals": ["8.8871640e-01+0.3681184j", "7.3223300e-02-0.17677669j",
                     "np.arange(4).reshape(2, 2)"],
    },
}

FILES = {
    "util_qsim_two_term": "tensorflow_quantum/core/src/util_qsim_test.cc",
    "util_qsim_identity": "tensorflow_quantum/core/src/util_qsim_test.cc",
    "adj_grad": "tensorflow_quantum/core/ops/tfq_adj_grad_op_test.py",
    "gradient_gates": "tensorflow_quantum/core/src/adj_util_test.cc",
    "padding": "tensorflow_quantum/core/ops/tfq_simulate_ops_test.py",
    "inner_product": "tensorflow_quantum/core/ops/math_ops/inner_product_op.py",
}


def verify_against_reference():
    if not REF:
        return None
    missing = []
    for key, rel in FILES.items():
        path = os.path.join(REF, rel)
        if not os.path.exists(path):
            return None
        text = open(path).read()
        for lit in GOLDENS[key]["literals"]:
            if lit not in text:
                missing.append((key, lit))
    return missing


def main():
    res = verify_against_reference()
    if res:
        raise SystemExit(f"literals not found in the reference: {res}")
    out = os.path.join(HERE, "reference_goldens.json")
    with open(out, "w") as f:
        json.dump(GOLDENS, f, indent=1)
    print("wrote", out, "(verified against reference)" if res == [] else "")


if __name__ == "__main__":
    main()
