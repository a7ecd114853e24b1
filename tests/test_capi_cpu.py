"""The C ABI without a GPU: the library loads, exports every symbol the public
header declares, and the host half (parse, resolve, validate) behaves like the
reference's Compute() preamble.  No kernel is launched here."""

import os
import re

import numpy as np
import pytest

from quantum_gb300 import _native, ops
from quantum_gb300 import serialize as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "tfq_gb300.h")).read()
    return sorted(set(re.findall(r"\b(tfqg_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _native.lib()
    names = _declared()
    assert len(names) >= 12
    for name in names:
        assert hasattr(lib, name), name
    assert set(_native.EXPORTED) <= set(names)


def test_version():
    assert b"sm_103a" in _native.lib().tfqg_version()


def _prog(ops_):
    return S.serialize_circuit(S.Circuit([[o] for o in ops_]))


Q = S.GridQubit.rect(1, 3)


@pytest.mark.parametrize("programs,names,psums,kind,pattern", [
    ([b"\xff\xff"], [], None, 0, "Unparseable proto"),
    ([_prog([S.XPow(Q[0], S.Symbol("a"))])], ["b"], None, 0,
     "Could not find symbol in parameter map: a"),
    ([_prog([S.depolarize(Q[0], 0.1)])], [], None, 0, "cirq.Channel"),
    ([_prog([S.X(Q[0])])], [],
     [[S.serialize_paulisum([(1.0, [(Q[2], "Z")])])]], 0,
     "Pauli sum operating on qubits not found"),
    ([S.serialize_circuit(S.Circuit([[S.Operation("ZZZ", {}, [Q[0]])]]))], [],
     None, 0, "Could not parse gate id: ZZZ"),
    ([S.serialize_circuit(S.Circuit([[S.Operation("XP", {"exponent": ("float", 1.0)},
                                                  [Q[0]])]]))], [], None, 0,
     "Could not find arg: exponent_scalar in op."),
    ([S.serialize_circuit(S.Circuit([[S.Operation("XP", {}, [S.LineQubit(0)])
                                      .controlled_by(Q[1])]]))], [], None, 0,
     "Could not find arg"),
    ([S.serialize_circuit(S.Circuit([[S.Operation("FOO", {}, [Q[0]])]]))], [], None, 2,
     "Could not parse channel id: FOO"),
])
def test_host_validation_errors(programs, names, psums, kind, pattern):
    with pytest.raises(_native.InvalidArgumentError, match=pattern):
        ops.Batch(programs, names, psums, kind)


def test_unparseable_qubit():
    op = S.X(Q[0])
    op.qubits = [type("Q", (), {"id": "a_b"})()]
    with pytest.raises(_native.InvalidArgumentError, match="Unable to parse qubit: a_b"):
        ops.Batch([S.serialize_circuit(S.Circuit([[op]]))], [], None)


def test_mismatched_controls():
    op = S.X(Q[0])
    op.args["control_qubits"] = ("string", "0_1,0_2")
    op.args["control_values"] = ("string", "1")
    with pytest.raises(_native.InvalidArgumentError, match="Mistmatched number"):
        ops.Batch([S.serialize_circuit(S.Circuit([[op]]))], [], None)


def test_shape_checks_match_reference_messages():
    p = _prog([S.X(Q[0])])
    b = ops.Batch([p], ["a"], [[S.serialize_paulisum([(1.0, [(Q[0], "Z")])])]])
    with pytest.raises(_native.InvalidArgumentError,
                       match="symbol names and value sizes do not match"):
        b.expectation(np.zeros((1, 2), np.float32))
    with pytest.raises(_native.InvalidArgumentError,
                       match="Number of circuits and symbol_values do not match"):
        b.expectation(np.zeros((2, 1), np.float32))
    with pytest.raises(_native.InvalidArgumentError, match="must be rank 2"):
        b.expectation(np.zeros((3,), np.float32))
    with pytest.raises(_native.InvalidArgumentError, match="programs must be rank 1"):
        ops.Batch([[p]], [], None)
    with pytest.raises(_native.InvalidArgumentError, match="pauli_sums must be rank 2"):
        ops.Batch([p], [], [b"x"])


def test_max_num_qubits_and_resolution_order():
    line = S.LineQubit.range(3)
    p1 = _prog([S.X(line[0]), S.CNOT(line[1], line[2])])
    p2 = _prog([S.X(Q[0])])
    empty = S.serialize_circuit(S.Circuit())
    b = ops.Batch([p1, p2, empty], [], None)
    assert b.max_num_qubits == 3
    assert ops.Batch([empty], [], None).max_num_qubits == 0


def test_empty_batch():
    b = ops.Batch([], [], np.zeros((0, 0), dtype=object).tolist() or
                  np.empty((0, 0), dtype=object))
    assert b.batch_size == 0


def test_sampled_expectation_input_checks():
    """tfq_simulate_ops_test.py sampled-expectation input checks: rank and
    dimension messages, and num_samples elements >= 1 (parse_context.cc:
    349-381), raised before any GPU work."""
    prog = _prog([S.HPow(Q[0]), S.I(Q[1])])
    ps = S.serialize_paulisum([(1.0, [(Q[0], "Z")])])
    b = ops.Batch([prog], [], [[ps]])
    with pytest.raises(_native.InvalidArgumentError, match="num_samples must be rank 2"):
        b.sampled_expectation(np.zeros((1, 0), np.float32), [1])
    with pytest.raises(_native.InvalidArgumentError,
                       match="Dimension 0 of num_samples and pauli_sums do not match"):
        b.sampled_expectation(np.zeros((1, 0), np.float32), [[1], [1]])
    with pytest.raises(_native.InvalidArgumentError,
                       match="Dimension 1 of num_samples and pauli_sums do not match"):
        b.sampled_expectation(np.zeros((1, 0), np.float32), [[1, 1]])
    with pytest.raises(_native.InvalidArgumentError,
                       match="Each element of num_samples must be greater than 0"):
        b.sampled_expectation(np.zeros((1, 0), np.float32), [[0]])


def test_inner_product_input_checks():
    """tfq_inner_product's resolution and parse errors (program_resolution.cc:
    188-310, math_ops/tfq_inner_product.cc:48-166), raised at batch creation
    without a GPU."""
    q = S.GridQubit.rect(1, 3)
    ref = _prog([S.HPow(q[0]), S.HPow(q[1])])
    same = _prog([S.X(q[0]), S.X(q[1])])
    extra = _prog([S.X(q[0]), S.X(q[2])])
    fewer = _prog([S.X(q[0])])
    sym = _prog([S.XPow(q[0], S.Symbol("a")), S.X(q[1])])
    ops.InnerProductBatch([ref], [], [[same]])  # fine
    with pytest.raises(_native.InvalidArgumentError,
                       match="A paired circuit contains qubits not found in reference circuit."):
        ops.InnerProductBatch([ref], [], [[extra]])
    with pytest.raises(_native.InvalidArgumentError,
                       match="A reference circuit contains qubits not found in paired circuit."):
        ops.InnerProductBatch([ref], [], [[fewer]])
    with pytest.raises(_native.InvalidArgumentError,
                       match="Found symbols in other_programs.No symbols are allowed"):
        ops.InnerProductBatch([ref], ["a"], [[sym]])
    with pytest.raises(_native.InvalidArgumentError, match="other_programs must be rank 2"):
        ops.InnerProductBatch([ref], [], [same])
    with pytest.raises(_native.InvalidArgumentError,
                       match="programs and other_programs batch dimension do not match"):
        ops.InnerProductBatch([ref, ref], [], [[same]])
    # an empty reference program skips its paired circuits' checks
    ops.InnerProductBatch([S.serialize_circuit(S.Circuit())], [], [[extra]])


def test_wide_row_rule_follows_the_batch():
    """Rows of 22+ qubits always run on the whole grid; a row of n = 17..21
    qubits too when the batch streams R <= 2^(n-14) rows (a wide pass keeps
    2^(n-13) tiles busy; in the queue R rows run side by side); 16-qubit
    rows never."""
    import numpy as np
    from quantum_gb300 import _native, ops
    from quantum_gb300 import serialize as S
    from tests.circuits import random_circuit
    rng = np.random.default_rng(1)

    def prog(n):
        return S.serialize_circuit(random_circuit(S.GridQubit.rect(1, n), 2, rng, []))

    p16, p18, p5 = prog(16), prog(18), prog(5)
    p20 = prog(20)
    cases = [([p18], 1), ([p16], 0), ([p18] * 70, 0), ([p18] + [p5] * 100, 1),
             ([p18] * 10 + [p16] * 60, 0), ([p18] * 16, 16), ([p18] * 17, 0),
             ([p20] * 40, 40), ([p20] + [p18] * 20, 1)]
    for progs, want in cases:
        b = ops.Batch(progs, [], None)
        assert _native.batch_wide_rows(b._h) == want, (len(progs), want)
        b.close()


def test_max_num_qubits_of_symbolic_programs_without_a_gpu():
    """tfqg_max_num_qubits decodes and resolves qubits only (symbols are bound
    later, as GetProgramsAndNumQubits does), so it needs no symbol values and
    no GPU."""
    import ctypes
    from quantum_gb300 import _native
    from quantum_gb300 import serialize as S
    progs = [S.serialize_circuit(S.Circuit([[S.rx(q, S.Symbol("a"))
                                             for q in S.GridQubit.rect(1, n)]]))
             for n in (3, 9, 5)]
    pp, pl, keep = _native.string_array(progs)
    f = _native.lib().tfqg_max_num_qubits
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    mq = ctypes.c_int32()
    assert f(pp, pl, 3, ctypes.byref(mq)) == 0 and mq.value == 9
    bad, bl, keep2 = _native.string_array([b"\x0a\x05garbage"])
    assert f(bad, bl, 1, ctypes.byref(mq)) == 3


def test_parallel_parse_reports_the_first_error_in_row_order():
    """Distinct programs are decoded, resolved and compiled on the host's
    cores; the error raised is still the one a row-order loop meets first."""
    import pytest
    from quantum_gb300 import _native, ops
    from quantum_gb300 import serialize as S
    progs = []
    for i in range(64):
        q = S.GridQubit.rect(1, 2 + i % 5)
        progs.append(S.serialize_circuit(S.Circuit([[S.rx(q[0], 0.1 * (i + 1))],
                                                    [S.CNOT(q[0], q[1])]])))
    bad = list(progs)
    bad[50] = b"not a proto A"
    bad[20] = b"not a proto B"
    with pytest.raises(_native.InvalidArgumentError, match="not a proto B"):
        ops.Batch(bad, [], None)
    bad = list(progs)
    q = S.GridQubit.rect(1, 2)
    bad[45] = S.serialize_circuit(S.Circuit([[S.rx(q[0], S.Symbol("late"))]]))
    bad[30] = S.serialize_circuit(S.Circuit([[S.rx(q[1], S.Symbol("early"))]]))
    with pytest.raises(_native.InvalidArgumentError, match="early"):
        ops.Batch(bad, ["x"], None)
