"""Cirq-free builder and encoder for TFQ's serialized circuits and Pauli sums.

TFQ's ops take `tf.string` tensors holding binary `tfq.proto.Program` and
`tfq.proto.PauliSum` messages (tensorflow_quantum/core/proto/program.proto,
pauli_sum.proto).  TFQ produces them from cirq objects in
tensorflow_quantum/core/serialize/serializer.py; this module produces the
same wire bytes without cirq or the protobuf runtime, so synthetic circuits
can be built on machines that have neither.

Encoding rules kept identical to the reference serializer because the
simulator's results depend on them:

* a numeric exponent is rounded to 6 decimals (serializer.py:33-34 `_round`,
  used by `_symbol_extractor` serializer.py:87-116) and its scalar is 1.0;
* a symbolic exponent `s * Symbol` is written as `symbol=name` with
  `exponent_scalar=round(s, 6)` (serializer.py:52-84);
* `rx/ry/rz(theta)` are `X/Y/ZPowGate(exponent=theta/pi, global_shift=-0.5)`,
  so a symbolic angle carries the scalar round(1/pi, 6) = 0.31831;
* every gate carries `control_qubits` / `control_values` strings, empty when
  the gate is not controlled (serializer.py:119-131);
* qubit ids are "row_col" for grid qubits and "x" for line qubits
  (op_serializer.py:33-39);
* Pauli terms list their qubits sorted (serializer.py:925).
"""

import math
import struct

import numpy as np

__all__ = [
    "GridQubit", "LineQubit", "Symbol", "Operation", "Circuit",
    "serialize_circuit", "serialize_paulisum", "PauliTerm",
]


# --------------------------------------------------------------------------
# protobuf wire-format primitives (proto3, little-endian)
# --------------------------------------------------------------------------

def _varint(v):
    v = int(v)
    if v < 0:
        v += 1 << 64
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        if v:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _tag(field, wire_type):
    return _varint((field << 3) | wire_type)


def _ld(field, payload):
    """Length-delimited field (wire type 2)."""
    return _tag(field, 2) + _varint(len(payload)) + payload


def _str(field, s):
    return _ld(field, s.encode("utf-8"))


def _f32(field, x):
    return _tag(field, 5) + struct.pack("<f", float(x))


def _vint(field, v):
    return _tag(field, 0) + _varint(v)


# --------------------------------------------------------------------------
# qubits, symbols, parameters
# --------------------------------------------------------------------------

class GridQubit:
    __slots__ = ("row", "col")

    def __init__(self, row, col):
        self.row, self.col = int(row), int(col)

    @property
    def id(self):
        return f"{self.row}_{self.col}"

    def _key(self):
        return (self.row, self.col)

    def __lt__(self, other):
        return _qubit_sort_key(self) < _qubit_sort_key(other)

    def __eq__(self, other):
        return isinstance(other, GridQubit) and self._key() == other._key()

    def __hash__(self):
        return hash(("g", self.row, self.col))

    def __repr__(self):
        return f"GridQubit({self.row}, {self.col})"

    @staticmethod
    def rect(rows, cols, top=0, left=0):
        return [GridQubit(top + r, left + c) for r in range(rows)
                for c in range(cols)]


class LineQubit:
    __slots__ = ("x",)

    def __init__(self, x):
        self.x = int(x)

    @property
    def id(self):
        return f"{self.x}"

    def __lt__(self, other):
        return _qubit_sort_key(self) < _qubit_sort_key(other)

    def __eq__(self, other):
        return isinstance(other, LineQubit) and self.x == other.x

    def __hash__(self):
        return hash(("l", self.x))

    def __repr__(self):
        return f"LineQubit({self.x})"

    @staticmethod
    def range(n):
        return [LineQubit(i) for i in range(n)]


def _qubit_sort_key(q):
    # cirq sorts LineQubits before GridQubits by type name; within a type by
    # coordinates.  Only used to order the qubits of a Pauli term.
    if isinstance(q, LineQubit):
        return (0, q.x, 0)
    return (1, q.row, q.col)


class Symbol:
    """A named parameter, optionally multiplied by a scalar (`2.0 * s`)."""
    __slots__ = ("name", "scalar")

    def __init__(self, name, scalar=1.0):
        self.name = str(name)
        self.scalar = float(scalar)

    def __mul__(self, k):
        return Symbol(self.name, self.scalar * float(k))

    __rmul__ = __mul__

    def __truediv__(self, k):
        return Symbol(self.name, self.scalar / float(k))

    def __repr__(self):
        return f"Symbol({self.name!r}, {self.scalar})"


def _round6(x):
    return float(np.round(float(x), 6))


def _param_args(name, value):
    """Encode `name` and `name_scalar` args the way the reference does."""
    if isinstance(value, Symbol):
        scalar = 1.0 if value.scalar == 1.0 else _round6(value.scalar)
        return {name: ("symbol", value.name), name + "_scalar": ("float", scalar)}
    return {name: ("float", _round6(value)), name + "_scalar": ("float", 1.0)}


# --------------------------------------------------------------------------
# operations
# --------------------------------------------------------------------------

class Operation:
    """One serialized operation: gate id, args map, qubits."""
    __slots__ = ("gate_id", "args", "qubits")

    def __init__(self, gate_id, args, qubits):
        self.gate_id = gate_id
        self.args = dict(args)
        self.qubits = list(qubits)
        self.args.setdefault("control_qubits", ("string", ""))
        self.args.setdefault("control_values", ("string", ""))

    def controlled_by(self, *controls, control_values=None):
        """Return this op controlled by `controls` (values default to 1)."""
        controls = list(controls)
        if control_values is None:
            control_values = [1] * len(controls)
        args = dict(self.args)
        args["control_qubits"] = ("string", ",".join(q.id for q in controls))
        args["control_values"] = ("string",
                                  ",".join(str(int(v)) for v in control_values))
        return Operation(self.gate_id, args, self.qubits)

    def encode(self):
        out = _ld(1, _str(1, self.gate_id))
        for key in sorted(self.args):
            kind, val = self.args[key]
            if kind == "symbol":
                arg = _str(2, val)
            elif kind == "float":
                arg = _ld(1, _f32(1, val))
            elif kind == "string":
                arg = _ld(1, _str(3, val))
            else:
                raise ValueError(f"unknown arg kind {kind}")
            entry = _str(1, key) + _ld(2, arg)
            out += _ld(2, entry)
        for q in self.qubits:
            out += _ld(3, _str(2, q.id))
        return out

    def __repr__(self):
        return f"Operation({self.gate_id}, {self.qubits})"


def _eigen(gate_id, qubits, exponent, global_shift):
    args = _param_args("exponent", exponent)
    args["global_shift"] = ("float", float(global_shift))
    return Operation(gate_id, args, qubits)


# Eigen gates G**t with global shift (serializer.py:456-485 / 738-750).
def XPow(q, exponent=1.0, global_shift=0.0):
    return _eigen("XP", [q], exponent, global_shift)


def YPow(q, exponent=1.0, global_shift=0.0):
    return _eigen("YP", [q], exponent, global_shift)


def ZPow(q, exponent=1.0, global_shift=0.0):
    return _eigen("ZP", [q], exponent, global_shift)


def HPow(q, exponent=1.0, global_shift=0.0):
    return _eigen("HP", [q], exponent, global_shift)


def XXPow(q0, q1, exponent=1.0, global_shift=0.0):
    return _eigen("XXP", [q0, q1], exponent, global_shift)


def YYPow(q0, q1, exponent=1.0, global_shift=0.0):
    return _eigen("YYP", [q0, q1], exponent, global_shift)


def ZZPow(q0, q1, exponent=1.0, global_shift=0.0):
    return _eigen("ZZP", [q0, q1], exponent, global_shift)


def CZPow(q0, q1, exponent=1.0, global_shift=0.0):
    return _eigen("CZP", [q0, q1], exponent, global_shift)


def CNotPow(q0, q1, exponent=1.0, global_shift=0.0):
    return _eigen("CNP", [q0, q1], exponent, global_shift)


def SwapPow(q0, q1, exponent=1.0, global_shift=0.0):
    return _eigen("SP", [q0, q1], exponent, global_shift)


def ISwapPow(q0, q1, exponent=1.0, global_shift=0.0):
    return _eigen("ISP", [q0, q1], exponent, global_shift)


def _angle_exponent(theta):
    # rx(theta) == XPowGate(exponent=theta/pi, global_shift=-0.5)
    if isinstance(theta, Symbol):
        return theta / math.pi
    return float(theta) / math.pi


def rx(q, theta):
    return XPow(q, _angle_exponent(theta), -0.5)


def ry(q, theta):
    return YPow(q, _angle_exponent(theta), -0.5)


def rz(q, theta):
    return ZPow(q, _angle_exponent(theta), -0.5)


def X(q):
    return XPow(q)


def Y(q):
    return YPow(q)


def Z(q):
    return ZPow(q)


def H(q):
    return HPow(q)


def CZ(q0, q1):
    return CZPow(q0, q1)


def CNOT(q0, q1):
    return CNotPow(q0, q1)


def SWAP(q0, q1):
    return SwapPow(q0, q1)


def ISWAP(q0, q1):
    return ISwapPow(q0, q1)


def PhasedXPow(q, phase_exponent, exponent=1.0, global_shift=0.0):
    args = _param_args("phase_exponent", phase_exponent)
    args.update(_param_args("exponent", exponent))
    args["global_shift"] = ("float", float(global_shift))
    return Operation("PXP", args, [q])


def PhasedISwapPow(q0, q1, phase_exponent=0.25, exponent=1.0):
    args = _param_args("phase_exponent", phase_exponent)
    args.update(_param_args("exponent", exponent))
    args["global_shift"] = ("float", 0.0)
    return Operation("PISP", args, [q0, q1])


def FSim(q0, q1, theta, phi):
    args = _param_args("theta", theta)
    args.update(_param_args("phi", phi))
    return Operation("FSIM", args, [q0, q1])


def I(q):
    return Operation("I", {"unused": ("float", 1.0)}, [q])


# Channels (serializer.py:175-452).
def depolarize(q, p):
    return Operation("DP", {"p": ("float", p)}, [q])


def asymmetric_depolarize(q, p_x, p_y, p_z):
    return Operation("ADP", {"p_x": ("float", p_x), "p_y": ("float", p_y),
                             "p_z": ("float", p_z)}, [q])


def generalized_amplitude_damp(q, p, gamma):
    return Operation("GAD", {"p": ("float", p), "gamma": ("float", gamma)}, [q])


def amplitude_damp(q, gamma):
    return Operation("AD", {"gamma": ("float", gamma)}, [q])


def reset(q):
    return Operation("RST", {}, [q])


def phase_damp(q, gamma):
    return Operation("PD", {"gamma": ("float", gamma)}, [q])


def phase_flip(q, p):
    return Operation("PF", {"p": ("float", p)}, [q])


def bit_flip(q, p):
    return Operation("BF", {"p": ("float", p)}, [q])


# --------------------------------------------------------------------------
# circuits and Pauli sums
# --------------------------------------------------------------------------

class Circuit:
    """A list of moments; each moment is a list of Operations."""

    def __init__(self, moments=None):
        self.moments = [list(m) for m in (moments or [])]

    def append_moment(self, ops):
        self.moments.append(list(ops))
        return self

    def append(self, op):
        """Append `op` in its own moment."""
        self.moments.append([op])
        return self

    @property
    def all_qubits(self):
        qs = set()
        for m in self.moments:
            for op in m:
                qs.update(op.qubits)
        return qs


def serialize_circuit(circuit):
    """Encode a Circuit as a binary tfq.proto.Program."""
    circ = _vint(1, 1)  # scheduling_strategy = MOMENT_BY_MOMENT
    for moment in circuit.moments:
        mom = b"".join(_ld(1, op.encode()) for op in moment)
        circ += _ld(2, mom)
    lang = _str(1, "tfq_gate_set")
    return _ld(1, lang) + _ld(2, circ)


class PauliTerm:
    """coefficient * prod_k P_k(q_k) with P in {'X','Y','Z'}."""

    def __init__(self, coefficient, paulis):
        self.coefficient = complex(coefficient)
        self.paulis = sorted(((q, str(p)) for q, p in paulis),
                             key=lambda qp: _qubit_sort_key(qp[0]))

    def encode(self):
        out = b""
        if self.coefficient.real != 0.0:
            out += _f32(1, self.coefficient.real)
        if self.coefficient.imag != 0.0:
            out += _f32(2, self.coefficient.imag)
        for q, p in self.paulis:
            out += _ld(3, _str(1, q.id) + _str(2, p))
        return out


def serialize_paulisum(terms):
    """Encode a list of PauliTerm (or (coef, [(qubit, 'X'), ...])) tuples."""
    out = b""
    for t in terms:
        if not isinstance(t, PauliTerm):
            t = PauliTerm(*t)
        out += _ld(1, t.encode())
    return out
