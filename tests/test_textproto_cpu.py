"""Text-format protos: the reference falls back to protobuf TextFormat when
a program or pauli sum is not binary (ParseProto, parse_context.cc:155-170).
The same circuits and sums given as binary and as text compile to identical
host tables (fingerprint of the packed tables); malformed text fails with the
reference's "Unparseable proto" error.  No GPU needed."""

import ctypes

import numpy as np
import pytest

from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S
from tests import textfmt
from tests.circuits import CHANNELS, random_circuit, random_paulisum


def _fingerprint(b):
    f = _native.lib().tfqg_internal_batch_fingerprint
    f.argtypes = [ctypes.c_void_p]
    f.restype = ctypes.c_uint64
    return f(b._h)


def _case(seed, n, channels=()):
    rng = np.random.default_rng(seed)
    qs = S.GridQubit.rect(1, n)
    names = ["a", "b", "c"]
    c = random_circuit(qs, 6, rng, names, p_control=0.3, channels=list(channels),
                       p_channel=0.3 if channels else 0.0)
    return (S.serialize_circuit(c), names,
            [random_paulisum(qs, rng), random_paulisum(qs, rng)])


@pytest.mark.parametrize("style", ["braces", "angles"])
@pytest.mark.parametrize("kind", [ops.KIND_FORWARD, ops.KIND_ADJOINT])
def test_text_and_binary_compile_identically(style, kind):
    progs, sums, text_progs, text_sums = [], [], [], []
    for seed, n in [(1, 3), (2, 6), (3, 9)]:
        p, names, ps = _case(seed, n)
        progs.append(p)
        sums.append(ps)
        text_progs.append(textfmt.to_text(p, "Program", style=style).encode())
        text_sums.append([textfmt.to_text(x, "PauliSum", style=style).encode() for x in ps])
    a = ops.Batch(progs, names, sums, kind=kind)
    b = ops.Batch(text_progs, names, text_sums, kind=kind)
    mixed = ops.Batch([progs[0], text_progs[1], progs[2]], names,
                      [sums[0], text_sums[1], sums[2]], kind=kind)
    assert _fingerprint(a) == _fingerprint(b) == _fingerprint(mixed)


def test_noisy_programs_in_text():
    p, names, ps = _case(7, 4, channels=CHANNELS)
    a = ops.Batch([p], names, [ps], kind=ops.KIND_NOISY)
    b = ops.Batch([textfmt.to_text(p).encode()], names,
                  [[textfmt.to_text(x, "PauliSum").encode() for x in ps]], kind=ops.KIND_NOISY)
    assert _fingerprint(a) == _fingerprint(b)


HAND_WRITTEN = b"""
# a Hadamard on 0_0 and a symbolic X^t on 0_1, written by hand
language { gate_set: 'tfq_gate_set' }
circuit: {
  scheduling_strategy: 1
  moments: [
    { operations <
        gate { id: "H" "P" }                 # adjacent strings concatenate
        args { key: "exponent" value { arg_value { float_value: 1 } } },
        args { key: "exponent_scalar" value { arg_value { float_value: 1.0f } } };
        args { key: "global_shift" value { arg_value { float_value: 0.0 } } }
        args { key: "control_qubits" value { arg_value { string_value: "" } } }
        args { key: "control_values" value { arg_value { string_value: '' } } }
        qubits { id: "0_0" }
    > },
    { operations {
        gate { id: "XP" }
        args { key: "exponent" value { symbol: "t" } }
        args { key: "exponent_scalar" value { arg_value { float_value: 5e-1 } } }
        args { key: "global_shift" value { arg_value { float_value: .0 } } }
        args { key: "control_qubits" value { arg_value { string_value: "" } } }
        args { key: "control_values" value { arg_value { string_value: "" } } }
        qubits { id: "0_1" }
    } }
  ]
}
"""


def test_hand_written_text_matches_serializer():
    q = S.GridQubit.rect(1, 2)
    ref = S.serialize_circuit(S.Circuit([[S.HPow(q[0], 1.0)],
                                         [S.XPow(q[1], S.Symbol("t", 0.5))]]))
    ps = S.serialize_paulisum([(2.0, [(q[0], "Z"), (q[1], "X")])])
    text_ps = b'terms { coefficient_real: 2 paulis { qubit_id: "0_0" pauli_type: "Z" } ' \
              b'paulis: [ { qubit_id: "0_1" pauli_type: "X" } ] }'
    a = ops.Batch([ref], ["t"], [[ps]])
    b = ops.Batch([HAND_WRITTEN], ["t"], [[text_ps]])
    assert _fingerprint(a) == _fingerprint(b)


@pytest.mark.parametrize("bad", [
    b"circuit { moments { operations { gate { id: \"H\" } } }",  # unclosed
    b"circuit { no_such_field: 1 }",                              # unknown field
    b"circuit { moments { operations { gate { id: \"H } } } }",   # open string
    b"circuit { scheduling_strategy: NOT_A_STRATEGY }",           # bad enum
])
def test_malformed_text_is_unparseable(bad):
    with pytest.raises(_native.InvalidArgumentError, match="Unparseable proto"):
        ops.Batch([bad], [], None)
