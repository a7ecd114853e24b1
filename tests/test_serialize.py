"""The cirq-free encoder produces what the reference serializer would: checked
by decoding with the oracle's independent wire decoder."""

import math

import numpy as np

from oracle import tfq_oracle as O
from quantum_gb300 import serialize as S


def test_rx_symbol_scalar_and_shift():
    q = S.GridQubit(1, 2)
    m = O.decode_program(S.serialize_circuit(S.Circuit([[S.rx(q, S.Symbol("t"))]])))
    op = m[0][0]
    assert op["gate"] == "XP" and op["qubits"] == ["1_2"]
    assert op["args"]["exponent"]["symbol"] == "t"
    assert abs(op["args"]["exponent_scalar"]["float"] - np.float32(0.31831)) < 1e-7
    assert op["args"]["global_shift"]["float"] == np.float32(-0.5)
    assert op["args"]["control_qubits"]["string"] == ""


def test_numeric_exponent_rounded_to_6_decimals():
    q = S.LineQubit(4)
    m = O.decode_program(S.serialize_circuit(S.Circuit([[S.rz(q, 1.0)]])))
    assert m[0][0]["args"]["exponent"]["float"] == np.float32(round(1 / math.pi, 6))
    assert m[0][0]["qubits"] == ["4"]


def test_controls_encoded():
    q = S.GridQubit.rect(1, 3)
    op = S.FSim(q[0], q[1], S.Symbol("a") * 2.0, 0.5).controlled_by(q[2], control_values=[0])
    m = O.decode_program(S.serialize_circuit(S.Circuit([[op]])))
    a = m[0][0]["args"]
    assert a["control_qubits"]["string"] == "0_2"
    assert a["control_values"]["string"] == "0"
    assert a["theta_scalar"]["float"] == np.float32(2.0)


def test_paulisum_sorted_and_coefficients():
    q = S.GridQubit.rect(2, 2)
    t = O.decode_paulisum(S.serialize_paulisum([(0.5 - 0.25j, [(q[3], "X"), (q[0], "Z")])]))
    assert t[0]["re"] == np.float32(0.5) and t[0]["im"] == np.float32(-0.25)
    assert t[0]["paulis"] == [("0_0", "Z"), ("1_1", "X")]
