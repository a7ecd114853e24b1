"""Protobuf text format writer for tfq.proto Program / PauliSum wire bytes
(test fixtures: the same programs as binary and as text)."""

import struct

# message -> {field number: (name, type, sub-message)}
SCHEMA = {
    "Program": {1: ("language", "msg", "Language"), 2: ("circuit", "msg", "Circuit"),
                3: ("schedule", "msg", "Schedule")},
    "Circuit": {1: ("scheduling_strategy", "enum", None), 2: ("moments", "msg", "Moment")},
    "Moment": {1: ("operations", "msg", "Operation")},
    "Schedule": {3: ("scheduled_operations", "msg", "ScheduledOperation")},
    "ScheduledOperation": {1: ("operation", "msg", "Operation"),
                           2: ("start_time_picos", "int", None)},
    "Language": {1: ("gate_set", "str", None), 2: ("arg_function_language", "str", None)},
    "Operation": {1: ("gate", "msg", "Gate"), 2: ("args", "msg", "ArgsEntry"),
                  3: ("qubits", "msg", "Qubit")},
    "Gate": {1: ("id", "str", None)},
    "Qubit": {2: ("id", "str", None)},
    "ArgsEntry": {1: ("key", "str", None), 2: ("value", "msg", "Arg")},
    "Arg": {1: ("arg_value", "msg", "ArgValue"), 2: ("symbol", "str", None),
            3: ("func", "msg", "ArgFunction")},
    "ArgValue": {1: ("float_value", "float", None), 2: ("bool_values", "msg", "RepeatedBoolean"),
                 3: ("string_value", "str", None), 4: ("double_value", "double", None)},
    "RepeatedBoolean": {1: ("values", "bool", None)},
    "ArgFunction": {1: ("type", "str", None), 2: ("args", "msg", "Arg")},
    "PauliSum": {1: ("terms", "msg", "PauliTerm")},
    "PauliTerm": {1: ("coefficient_real", "float", None), 2: ("coefficient_imag", "float", None),
                  3: ("paulis", "msg", "PauliQubitPair")},
    "PauliQubitPair": {1: ("qubit_id", "str", None), 2: ("pauli_type", "str", None)},
}
ENUM = {0: "SCHEDULING_STRATEGY_UNSPECIFIED", 1: "MOMENT_BY_MOMENT"}


def _varint(b, i):
    v, s = 0, 0
    while True:
        c = b[i]
        i += 1
        v |= (c & 0x7F) << s
        s += 7
        if c < 0x80:
            return v, i


def _fields(b):
    i = 0
    while i < len(b):
        tag, i = _varint(b, i)
        fn, wt = tag >> 3, tag & 7
        if wt == 0:
            v, i = _varint(b, i)
        elif wt == 1:
            v, i = b[i:i + 8], i + 8
        elif wt == 2:
            n, i = _varint(b, i)
            v, i = b[i:i + n], i + n
        elif wt == 5:
            v, i = b[i:i + 4], i + 4
        else:
            raise ValueError("wire type")
        yield fn, v


def _quote(s):
    out = []
    for c in s:
        if c in b'"\\':
            out.append("\\" + chr(c))
        elif 32 <= c < 127:
            out.append(chr(c))
        else:
            out.append("\\%03o" % c)
    return '"' + "".join(out) + '"'


def to_text(b, message="Program", indent=0, style="braces"):
    """Text format of wire bytes `b`; style "angles" uses <...> bodies and
    ';' separators to exercise the other text syntax."""
    pad = "  " * indent
    lines = []
    for fn, v in _fields(bytes(b)):
        name, ty, sub = SCHEMA[message][fn]
        if ty == "msg":
            o, c = ("{", "}") if style == "braces" else ("<", ">")
            lines.append(f"{pad}{name} {o}")
            lines.append(to_text(v, sub, indent + 1, style))
            lines.append(f"{pad}{c}")
            continue
        if ty == "str":
            val = _quote(v)
        elif ty == "float":
            val = repr(struct.unpack("<f", v)[0])
        elif ty == "double":
            val = repr(struct.unpack("<d", v)[0])
        elif ty == "enum":
            val = ENUM[v]
        elif ty == "bool":
            val = "true" if v else "false"
        else:
            val = str(v)
        sep = "" if style == "braces" else ";"
        lines.append(f"{pad}{name}: {val}{sep}")
    return "\n".join(l for l in lines if l)
