"""CPU oracle for the TFQ state-vector hot path (TEST INFRASTRUCTURE ONLY).

This module is the checker, never the product: only tests, the smoke check
and the CPU-baseline leg of the benchmark may import it.  It restates, in
complex128 numpy, the algorithm of the reference ops:

* proto decode ............ tensorflow_quantum/core/ops/parse_context.cc:155-170
* qubit resolution ........ tensorflow_quantum/core/src/program_resolution.cc:49-186
* symbol maps ............. tensorflow_quantum/core/ops/parse_context.cc:405-461
* gate construction ....... tensorflow_quantum/core/src/circuit_parser_qsim.cc:53-596
  (qsim index = n-1-q, fp32 `exponent * exponent_scalar`)
* channels ................ circuit_parser_qsim.cc:598-769, noisy wrap :773-826
* expectation ............. tensorflow_quantum/core/src/util_qsim.h:142-188
* state padding ........... tensorflow_quantum/core/ops/tfq_simulate_state_op.cc:196-207
* sample bit layout ....... tensorflow_quantum/core/ops/tfq_simulate_samples_op.cc:226-243
* adjoint gradient ........ tensorflow_quantum/core/ops/tfq_adj_grad_op.cc:199-276,
  AccumulateOperators util_qsim.h:362-414, FD gradient gates
  tensorflow_quantum/core/src/adj_util.cc:32,175-302
* inner product ........... tensorflow_quantum/core/ops/math_ops/tfq_inner_product.cc,
  paired resolution program_resolution.cc:188-310, gradient
  math_ops/tfq_inner_product_grad.cc:216-318
* noisy expectation ....... tensorflow_quantum/core/ops/noise/tfq_noisy_expectation.cc
  (restated as an exact density-matrix evolution: the trajectory average
  converges to it)

The gate matrices follow the published definitions of the cirq gate families
(EigenGate: sum_k exp(i*pi*t*(lambda_k + s)) P_k), which the reference's
external simulator (qsim v0.21.0, not vendored) implements.  Parity of this
oracle is pinned by the reference's own known-answer tests, stored in
tests/golden/reference_goldens.json.
"""

import math
import struct

import numpy as np

F32 = np.float32
GRAD_EPS = F32(5e-3)  # adj_util.cc:32


class InvalidArgument(ValueError):
    """Mirrors tensorflow::errors::InvalidArgument."""


# ---------------------------------------------------------------------------
# protobuf wire decoding (Program / PauliSum)
# ---------------------------------------------------------------------------

def _read_varint(b, i):
    shift = 0
    v = 0
    while True:
        if i >= len(b) or shift > 63:
            raise InvalidArgument("bad varint")
        c = b[i]
        i += 1
        v |= (c & 0x7F) << shift
        if not c & 0x80:
            return v, i
        shift += 7


def _fields(b):
    """Yield (field_number, wire_type, value) for a serialized message."""
    i = 0
    n = len(b)
    while i < n:
        key, i = _read_varint(b, i)
        fn, wt = key >> 3, key & 7
        if fn == 0:
            raise InvalidArgument("bad field number")
        if wt == 0:
            v, i = _read_varint(b, i)
        elif wt == 1:
            if i + 8 > n:
                raise InvalidArgument("truncated")
            v = b[i:i + 8]
            i += 8
        elif wt == 2:
            ln, i = _read_varint(b, i)
            if i + ln > n:
                raise InvalidArgument("truncated")
            v = b[i:i + ln]
            i += ln
        elif wt == 5:
            if i + 4 > n:
                raise InvalidArgument("truncated")
            v = b[i:i + 4]
            i += 4
        else:
            raise InvalidArgument("unsupported wire type")
        yield fn, wt, v


def _decode_arg(b):
    arg = {"float": F32(0.0), "symbol": "", "string": ""}
    for fn, wt, v in _fields(b):
        if fn == 1 and wt == 2:  # ArgValue
            for fn2, wt2, v2 in _fields(v):
                if fn2 == 1 and wt2 == 5:
                    arg["float"] = F32(struct.unpack("<f", v2)[0])
                elif fn2 == 3 and wt2 == 2:
                    arg["string"] = v2.decode("utf-8")
        elif fn == 2 and wt == 2:
            arg["symbol"] = v.decode("utf-8")
    return arg


def _decode_op(b):
    op = {"gate": "", "args": {}, "qubits": []}
    for fn, wt, v in _fields(b):
        if fn == 1 and wt == 2:
            for fn2, wt2, v2 in _fields(v):
                if fn2 == 1 and wt2 == 2:
                    op["gate"] = v2.decode("utf-8")
        elif fn == 2 and wt == 2:
            key, val = "", b""
            for fn2, wt2, v2 in _fields(v):
                if fn2 == 1 and wt2 == 2:
                    key = v2.decode("utf-8")
                elif fn2 == 2 and wt2 == 2:
                    val = v2
            op["args"][key] = _decode_arg(val)
        elif fn == 3 and wt == 2:
            qid = ""
            for fn2, wt2, v2 in _fields(v):
                if fn2 == 2 and wt2 == 2:
                    qid = v2.decode("utf-8")
            op["qubits"].append(qid)
    return op


def decode_program(b):
    """Binary tfq.proto.Program -> list of moments (lists of op dicts)."""
    try:
        moments = []
        for fn, wt, v in _fields(bytes(b)):
            if fn == 2 and wt == 2:  # circuit
                for fn2, wt2, v2 in _fields(v):
                    if fn2 == 2 and wt2 == 2:
                        ops = []
                        for fn3, wt3, v3 in _fields(v2):
                            if fn3 == 1 and wt3 == 2:
                                ops.append(_decode_op(v3))
                        moments.append(ops)
        return moments
    except (InvalidArgument, UnicodeDecodeError):
        raise InvalidArgument("Unparseable proto: " + repr(b)) from None


def decode_paulisum(b):
    try:
        terms = []
        for fn, wt, v in _fields(bytes(b)):
            if fn == 1 and wt == 2:
                t = {"re": F32(0.0), "im": F32(0.0), "paulis": []}
                for fn2, wt2, v2 in _fields(v):
                    if fn2 == 1 and wt2 == 5:
                        t["re"] = F32(struct.unpack("<f", v2)[0])
                    elif fn2 == 2 and wt2 == 5:
                        t["im"] = F32(struct.unpack("<f", v2)[0])
                    elif fn2 == 3 and wt2 == 2:
                        qid, ptype = "", ""
                        for fn3, wt3, v3 in _fields(v2):
                            if fn3 == 1 and wt3 == 2:
                                qid = v3.decode("utf-8")
                            elif fn3 == 2 and wt3 == 2:
                                ptype = v3.decode("utf-8")
                        t["paulis"].append((qid, ptype))
                terms.append(t)
        return terms
    except (InvalidArgument, UnicodeDecodeError):
        raise InvalidArgument("Unparseable proto: " + repr(b)) from None


# ---------------------------------------------------------------------------
# qubit resolution (program_resolution.cc:49-186)
# ---------------------------------------------------------------------------

INT_MAX = 2147483647


def _atoi(s):
    s = s.strip()
    if not s or not (s.lstrip("+-").isdigit()):
        raise ValueError
    v = int(s)
    if v < -2**31 or v >= 2**31:
        raise ValueError
    return v


def _register(qb_string, ids):
    if not qb_string:
        return
    for qb in qb_string.split(","):
        parts = qb.split("_")
        if len(parts) == 1:
            parts = [str(INT_MAX)] + parts
        if len(parts) != 2:
            raise InvalidArgument("Unable to parse qubit: " + qb)
        try:
            r, c = _atoi(parts[0]), _atoi(parts[1])
        except ValueError:
            raise InvalidArgument("Unable to parse qubit: " + qb) from None
        ids.add(((r, c), qb))


def _control_str(op, key):
    a = op["args"].get(key)
    return a["string"] if a is not None else ""


def resolve(moments, psums=None):
    """Return (n, id->index) and raise on PauliSums naming unknown qubits."""
    if not moments:
        return 0, {}
    ids = set()
    for m in moments:
        for op in m:
            for q in op["qubits"]:
                _register(q, ids)
            _register(_control_str(op, "control_qubits"), ids)
    order = sorted(ids)
    index = {s: i for i, (_, s) in enumerate(order)}
    if psums is not None:
        for ps in psums:
            for t in ps:
                for qid, _ in t["paulis"]:
                    if qid not in index:
                        raise InvalidArgument(
                            "Found a Pauli sum operating on qubits not found "
                            "in circuit.")
    return len(order), index


# ---------------------------------------------------------------------------
# gate matrices (cirq big-endian: the first listed qubit is the MSB)
# ---------------------------------------------------------------------------

_I2 = np.eye(2, dtype=np.complex128)
_X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
_Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
_Z = np.diag([1, -1]).astype(np.complex128)
_Hm = np.array([[1, 1], [1, -1]], dtype=np.complex128) / math.sqrt(2)


def _eig(t, s, projs):
    """sum_k exp(i*pi*t*(lam_k + s)) P_k for (lam_k, P_k) in projs."""
    t = float(t)
    s = float(s)
    u = 0
    for lam, p in projs:
        u = u + np.exp(1j * math.pi * t * (lam + s)) * p
    return u


def _pauli_projs(P):
    d = P.shape[0]
    e = np.eye(d, dtype=np.complex128)
    return [(0.0, (e + P) / 2), (1.0, (e - P) / 2)]


def _cx_projs():
    p0 = np.zeros((4, 4), dtype=np.complex128)
    p1 = np.zeros((4, 4), dtype=np.complex128)
    p0[:2, :2] = _I2
    p0[2:, 2:] = (_I2 + _X) / 2
    p1[2:, 2:] = (_I2 - _X) / 2
    return [(0.0, p0), (1.0, p1)]


def _swap_projs(iswap=False):
    p00 = np.zeros((4, 4), dtype=np.complex128)
    p00[0, 0] = p00[3, 3] = 1
    sym = np.zeros((4, 4), dtype=np.complex128)
    sym[1, 1] = sym[2, 2] = sym[1, 2] = sym[2, 1] = 0.5
    anti = np.zeros((4, 4), dtype=np.complex128)
    anti[1, 1] = anti[2, 2] = 0.5
    anti[1, 2] = anti[2, 1] = -0.5
    if iswap:
        return [(0.0, p00), (0.5, sym), (-0.5, anti)]
    return [(0.0, p00 + sym), (1.0, anti)]


def eigen_matrix(gate_id, t, s):
    if gate_id == "XP":
        return _eig(t, s, _pauli_projs(_X))
    if gate_id == "YP":
        return _eig(t, s, _pauli_projs(_Y))
    if gate_id == "ZP":
        return _eig(t, s, _pauli_projs(_Z))
    if gate_id == "HP":
        return _eig(t, s, _pauli_projs(_Hm))
    if gate_id == "XXP":
        return _eig(t, s, _pauli_projs(np.kron(_X, _X)))
    if gate_id == "YYP":
        return _eig(t, s, _pauli_projs(np.kron(_Y, _Y)))
    if gate_id == "ZZP":
        return _eig(t, s, _pauli_projs(np.kron(_Z, _Z)))
    if gate_id == "CZP":
        p1 = np.zeros((4, 4), dtype=np.complex128)
        p1[3, 3] = 1
        return _eig(t, s, [(0.0, np.eye(4) - p1), (1.0, p1)])
    if gate_id == "CNP":
        return _eig(t, s, _cx_projs())
    if gate_id == "SP":
        return _eig(t, s, _swap_projs(False))
    if gate_id == "ISP":
        return _eig(t, s, _swap_projs(True))
    raise KeyError(gate_id)


def phased_x_matrix(p, t, s):
    z = np.diag([1, np.exp(1j * math.pi * float(p))])
    x = _eig(t, 0.0, _pauli_projs(_X))
    return (z @ x @ np.conj(z)) * np.exp(1j * math.pi * float(s) * float(t))


def fsim_matrix(theta, phi):
    c, s = math.cos(float(theta)), math.sin(float(theta))
    return np.array([[1, 0, 0, 0], [0, c, -1j * s, 0], [0, -1j * s, c, 0],
                     [0, 0, 0, np.exp(-1j * float(phi))]], dtype=np.complex128)


def phased_iswap_matrix(p, t):
    c, s = math.cos(math.pi * float(t) / 2), math.sin(math.pi * float(t) / 2)
    f = np.exp(2j * math.pi * float(p))
    return np.array([[1, 0, 0, 0], [0, c, 1j * s * f, 0],
                     [0, 1j * s * np.conj(f), c, 0], [0, 0, 0, 1]],
                    dtype=np.complex128)


EIGEN_1Q = ("XP", "YP", "ZP", "HP")
EIGEN_2Q = ("XXP", "YYP", "ZZP", "CZP", "CNP", "SP", "ISP")
GATE_IDS = ("I", "HP", "XP", "XXP", "YP", "YYP", "ZP", "ZZP", "CZP", "I2",
            "CNP", "SP", "ISP", "PXP", "FSIM", "PISP")
CHANNEL_IDS = ("DP", "ADP", "GAD", "AD", "RST", "PD", "PF", "BF")


class Gate:
    """A resolved gate: matrix on `qubits` (cirq order) with controls.

    `grads` lists (symbol_name, dmatrix) pairs for symbolic parameters in the
    order the reference appends them (adj_util.cc:37-150).
    """

    def __init__(self, gid, qubits, matrix, controls=(), cvals=(), grads=()):
        self.gid = gid
        self.qubits = list(qubits)
        self.matrix = matrix
        self.controls = list(controls)
        self.cvals = list(cvals)
        self.grads = list(grads)


def _arg(op, name, smap):
    """ParseProtoArg (circuit_parser_qsim.cc:53-82)."""
    a = op["args"].get(name)
    if a is None:
        raise InvalidArgument("Could not find arg: " + name + " in op.")
    val = a["float"]
    sym = None
    if a["symbol"]:
        if a["symbol"] not in smap:
            raise InvalidArgument(
                "Could not find symbol in parameter map: " + a["symbol"])
        val = smap[a["symbol"]]
        sym = a["symbol"]
    return F32(val), sym


def _controls(op, index):
    cq = _control_str(op, "control_qubits")
    cv = _control_str(op, "control_values")
    if cq == "" and cv == "":
        return [], []
    qt = cq.split(",")
    vt = cv.split(",")
    if len(qt) != len(vt):
        raise InvalidArgument(
            "Mistmatched number of control qubits and control values.")
    qs = [index[t] for t in qt]
    vs = []
    for t in vt:
        try:
            vs.append(_atoi(t))
        except ValueError:
            raise InvalidArgument("Unparseable control value: " + t) from None
    return qs, vs


def _fd(make, x, scale):
    """FD gradient gate (adj_util.cc:175-186): (G(x+eps)-G(x-eps))*0.5/eps.

    Parameters are combined in fp32 exactly as the reference does."""
    hi = make(F32(F32(x + GRAD_EPS) * scale))
    lo = make(F32(F32(x - GRAD_EPS) * scale))
    return (hi - lo) * (0.5 / float(GRAD_EPS))


def _analytic(make, x, scale, h=1e-6):
    """Exact derivative d/dx G(x*scale) by a complex128 central difference
    with a tiny step (error ~h^2)."""
    xs = float(x) * float(scale)
    return (make(xs + h * float(scale)) - make(xs - h * float(scale))) / (2 * h)


def build_gate(op, index, smap, grad_rule="fd"):
    """Gate construction (circuit_parser_qsim.cc:154-596)."""
    gid = op["gate"]
    qubits = [index[q] for q in op["qubits"]]
    dmake = _fd if grad_rule == "fd" else _analytic
    grads = []
    if gid in ("I", "I2"):
        m = np.eye(2 ** len(qubits), dtype=np.complex128)
    elif gid in EIGEN_1Q or gid in EIGEN_2Q:
        e, esym = _arg(op, "exponent", smap)
        es, _ = _arg(op, "exponent_scalar", smap)
        gs, _ = _arg(op, "global_shift", smap)
        m = eigen_matrix(gid, F32(e * es), gs)
        if esym is not None:
            grads.append((esym, dmake(lambda t: eigen_matrix(gid, t, gs), e, es)))
    elif gid == "PXP":
        e, esym = _arg(op, "exponent", smap)
        es, _ = _arg(op, "exponent_scalar", smap)
        p, psym = _arg(op, "phase_exponent", smap)
        ps, _ = _arg(op, "phase_exponent_scalar", smap)
        gs, _ = _arg(op, "global_shift", smap)
        pe, te = F32(p * ps), F32(e * es)
        m = phased_x_matrix(pe, te, gs)
        # phase exponent first, then exponent (circuit_parser_qsim.cc:436-445)
        if psym is not None:
            grads.append((psym, dmake(lambda x: phased_x_matrix(x, te, gs), p, ps)))
        if esym is not None:
            grads.append((esym, dmake(lambda x: phased_x_matrix(pe, x, gs), e, es)))
    elif gid == "FSIM":
        th, thsym = _arg(op, "theta", smap)
        ths, _ = _arg(op, "theta_scalar", smap)
        ph, phsym = _arg(op, "phi", smap)
        phs, _ = _arg(op, "phi_scalar", smap)
        te, pe = F32(th * ths), F32(ph * phs)
        m = fsim_matrix(te, pe)
        if thsym is not None:
            grads.append((thsym, dmake(lambda x: fsim_matrix(x, pe), th, ths)))
        if phsym is not None:
            grads.append((phsym, dmake(lambda x: fsim_matrix(te, x), ph, phs)))
    elif gid == "PISP":
        e, esym = _arg(op, "exponent", smap)
        es, _ = _arg(op, "exponent_scalar", smap)
        p, psym = _arg(op, "phase_exponent", smap)
        ps, _ = _arg(op, "phase_exponent_scalar", smap)
        pe, te = F32(p * ps), F32(e * es)
        m = phased_iswap_matrix(pe, te)
        if psym is not None:
            grads.append((psym, dmake(lambda x: phased_iswap_matrix(x, te), p, ps)))
        if esym is not None:
            grads.append((esym, dmake(lambda x: phased_iswap_matrix(pe, x), e, es)))
    else:
        raise InvalidArgument(
            "Could not parse gate id: " + gid + ". This is likely because a "
            "cirq.Channel was used in an op that does not support them.")
    cq, cv = _controls(op, index)
    return Gate(gid, qubits, m, cq, cv, grads)


def channel_kraus(op):
    """Kraus operators of the supported channels (circuit_parser_qsim.cc:598-769;
    definitions of cirq's depolarize, asymmetric_depolarize,
    generalized_amplitude_damp, amplitude_damp, reset, phase_damp,
    phase_flip, bit_flip)."""
    gid = op["gate"]

    def f(name):
        a = op["args"].get(name)
        if a is None:
            raise InvalidArgument("Could not find arg: " + name + " in op.")
        return float(a["float"])

    if gid == "DP":
        p = f("p")
        return [math.sqrt(1 - p) * _I2] + [math.sqrt(p / 3) * P for P in (_X, _Y, _Z)]
    if gid == "ADP":
        px, py, pz = f("p_x"), f("p_y"), f("p_z")
        return [math.sqrt(1 - px - py - pz) * _I2, math.sqrt(px) * _X,
                math.sqrt(py) * _Y, math.sqrt(pz) * _Z]
    if gid == "GAD":
        p, g = f("p"), f("gamma")
        return [math.sqrt(p) * np.array([[1, 0], [0, math.sqrt(1 - g)]]),
                math.sqrt(p) * np.array([[0, math.sqrt(g)], [0, 0]]),
                math.sqrt(1 - p) * np.array([[math.sqrt(1 - g), 0], [0, 1]]),
                math.sqrt(1 - p) * np.array([[0, 0], [math.sqrt(g), 0]])]
    if gid == "AD":
        g = f("gamma")
        return [np.array([[1, 0], [0, math.sqrt(1 - g)]]),
                np.array([[0, math.sqrt(g)], [0, 0]])]
    if gid == "RST":
        return [np.array([[1, 0], [0, 0]]), np.array([[0, 1], [0, 0]])]
    if gid == "PD":
        g = f("gamma")
        return [np.array([[1, 0], [0, math.sqrt(1 - g)]]),
                np.array([[0, 0], [0, math.sqrt(g)]])]
    if gid == "PF":
        p = f("p")
        return [math.sqrt(1 - p) * _I2, math.sqrt(p) * _Z]
    if gid == "BF":
        p = f("p")
        return [math.sqrt(1 - p) * _I2, math.sqrt(p) * _X]
    raise InvalidArgument("Could not parse channel id: " + gid)


# ---------------------------------------------------------------------------
# state-vector arithmetic (complex128, axis q = qubit q, axis 0 = MSB)
# ---------------------------------------------------------------------------

def apply_matrix(psi, n, m, qubits, controls=(), cvals=()):
    """Return m (on `qubits`, first = MSB of m) applied to psi [2]*n."""
    k = len(qubits)
    psi = psi.reshape([2] * n)
    if controls:
        sl = [slice(None)] * n
        for c, v in zip(controls, cvals):
            sl[c] = int(v)
        sl = tuple(sl)
        sub = psi[sl]
        # axes of the remaining sub-array
        rest = [q for q in range(n) if q not in controls]
        sub_q = [rest.index(q) for q in qubits]
        out = psi.copy()
        out[sl] = apply_matrix(sub, len(rest), m, sub_q)
        return out
    mt = m.reshape([2] * (2 * k))
    out = np.tensordot(mt, psi, axes=(list(range(k, 2 * k)), qubits))
    # tensordot puts the gate's output axes first; move them back
    return np.moveaxis(out, list(range(k)), qubits)


def simulate(gates, n):
    psi = np.zeros([2] * n, dtype=np.complex128)
    psi[(0,) * n] = 1.0
    for g in gates:
        psi = apply_matrix(psi, n, g.matrix, g.qubits, g.controls, g.cvals)
    return psi


_PAULI = {"X": _X, "Y": _Y, "Z": _Z}


def apply_pauli_term(psi, n, paulis, index):
    for qid, p in paulis:
        psi = apply_matrix(psi, n, _PAULI[p], [index[qid]])
    return psi


def expectation(psi, n, terms, index):
    """ComputeExpectationQsim (util_qsim.h:142-188): sum_t Re(c_t)<psi|P_t|psi>."""
    v = 0.0
    for t in terms:
        if not t["paulis"]:
            v += float(t["re"])
            continue
        phi = apply_pauli_term(psi, n, t["paulis"], index)
        v += float(t["re"]) * float(np.real(np.vdot(psi, phi)))
    return v


# ---------------------------------------------------------------------------
# batched ops with the reference signatures
# ---------------------------------------------------------------------------

def _symbol_maps(symbol_names, symbol_values):
    vals = np.asarray(symbol_values, dtype=np.float32)
    if vals.ndim != 2:
        raise InvalidArgument("symbol_values must be rank 2. Got rank %d." % vals.ndim)
    if len(symbol_names) != vals.shape[1]:
        raise InvalidArgument("Input symbol names and value sizes do not match.")
    maps = []
    for row in vals:
        m = {}
        for j, name in enumerate(symbol_names):
            nm = name.decode() if isinstance(name, bytes) else name
            m[nm] = F32(row[j])
        maps.append(m)
    return maps


def _name_cols(symbol_names):
    cols = {}
    for j, name in enumerate(symbol_names):
        nm = name.decode() if isinstance(name, bytes) else name
        cols[nm] = j  # last column wins, like the reference's map assignment
    return cols


def _parse_all(programs, symbol_names, symbol_values, pauli_sums=None,
               grad_rule="fd", noisy=False):
    moms = [decode_program(p) for p in programs]
    psums = None
    if pauli_sums is not None:
        ps = np.asarray(pauli_sums, dtype=object)
        if ps.ndim != 2:
            raise InvalidArgument("pauli_sums must be rank 2. Got rank %d." % ps.ndim)
        psums = [[decode_paulisum(x) for x in row] for row in ps]
        if len(psums) != len(moms):
            raise InvalidArgument(
                "Number of circuits and PauliSums do not match. Got %d circuits "
                "and %d paulisums." % (len(moms), len(psums)))
    maps = _symbol_maps(symbol_names, symbol_values)
    if len(maps) != len(moms):
        raise InvalidArgument(
            "Number of circuits and symbol_values do not match. Got %d "
            "circuits and %d symbol values." % (len(moms), len(maps)))
    out = []
    for i, m in enumerate(moms):
        n, index = resolve(m, psums[i] if psums is not None else None)
        items = []
        if n > 0:
            for mom in m:
                for op in mom:
                    if noisy and op["gate"] not in GATE_IDS:
                        items.append(("channel", channel_kraus(op),
                                      [index[q] for q in op["qubits"]]))
                    else:
                        items.append(("gate", build_gate(op, index, maps[i],
                                                         grad_rule)))
        out.append((n, index, items))
    return out, psums


def simulate_expectation(programs, symbol_names, symbol_values, pauli_sums):
    parsed, psums = _parse_all(programs, symbol_names, symbol_values, pauli_sums)
    n_ops = np.asarray(pauli_sums, dtype=object).shape[1]
    out = np.zeros((len(parsed), n_ops), dtype=np.float64)
    for i, (n, index, items) in enumerate(parsed):
        gates = [g for _, g in items]
        if not gates:
            out[i, :] = -2.0
            continue
        psi = simulate(gates, n)
        for j in range(n_ops):
            out[i, j] = expectation(psi, n, psums[i][j], index)
    return out


def simulate_state(programs, symbol_names, symbol_values):
    parsed, _ = _parse_all(programs, symbol_names, symbol_values)
    maxn = max([p[0] for p in parsed], default=0)
    out = np.full((len(parsed), 2 ** maxn), -2 + 0j, dtype=np.complex128)
    for i, (n, index, items) in enumerate(parsed):
        if n == 0:
            out[i, 0] = 1.0
            continue
        psi = simulate([g for _, g in items], n)
        out[i, :2 ** n] = psi.reshape(-1)
    return out


def _check_paired(moments, index):
    """program_resolution.cc:253-307: a paired circuit uses exactly the
    reference circuit's qubits."""
    visited = set()
    for m in moments:
        for op in m:
            qs = list(op["qubits"])
            cs = _control_str(op, "control_qubits")
            if cs:
                qs += cs.split(",")
            for q in qs:
                if q not in index:
                    raise InvalidArgument("A paired circuit contains qubits not "
                                          "found in reference circuit.")
                visited.add(q)
    if len(visited) != len(index):
        raise InvalidArgument("A reference circuit contains qubits not found in "
                              "paired circuit.")


def inner_product(programs, symbol_names, symbol_values, other_programs):
    """tfq_inner_product (math_ops/tfq_inner_product.cc): out[i, j] =
    <psi_i(values_i) | phi_ij>, 1 for an empty reference program."""
    others = np.asarray(other_programs, dtype=object)
    if others.ndim != 2:
        raise InvalidArgument("other_programs must be rank 2. Got rank %d." % others.ndim)
    moms = [decode_program(p) for p in programs]
    other_moms = [[decode_program(x) for x in row] for row in others]
    if len(moms) != len(other_moms):
        raise InvalidArgument("programs and other_programs batch dimension do not "
                              "match. Foud: %d and %d" % (len(moms), len(other_moms)))
    resolved = []
    for i, m in enumerate(moms):
        n, index = resolve(m)
        if n > 0:
            for om in other_moms[i]:
                _check_paired(om, index)
        resolved.append((n, index))
    maps = _symbol_maps(symbol_names, symbol_values)
    gates = [[build_gate(op, idx, maps[i]) for mom in moms[i] for op in mom] if n else []
             for i, (n, idx) in enumerate(resolved)]
    out = np.zeros((len(moms), others.shape[1]), dtype=np.complex128)
    for i, (n, index) in enumerate(resolved):
        if not gates[i]:
            out[i, :] = 1.0
            continue
        psi = simulate(gates[i], n).reshape(-1)
        for j, om in enumerate(other_moms[i]):
            try:
                og = [build_gate(op, index, {}) for mom in om for op in mom]
            except (InvalidArgument, KeyError):
                raise InvalidArgument("Found symbols in other_programs.No symbols "
                                      "are allowed in these circuits.") from None
            phi = simulate(og, n).reshape(-1) if og else np.eye(1, 2 ** n, dtype=np.complex128)[0]
            out[i, j] = np.vdot(psi, phi)
    return out


def inner_product_grad(programs, symbol_names, symbol_values, other_programs,
                       downstream_grads):
    """TfqInnerProductGrad (math_ops/tfq_inner_product_grad.cc:216-318):
    out[i, p] = sum over the gates using symbol p of <dU psi_before | chi>,
    chi = sum_j g_ij |phi_ij> uncomputed alongside psi (FD gradient gates,
    control projector as in the adjoint op); complex, no factor 2."""
    others = np.asarray(other_programs, dtype=object)
    ref = inner_product(programs, symbol_names, symbol_values, other_programs)  # checks
    del ref
    parsed, _ = _parse_all(programs, symbol_names, symbol_values)
    cols = _name_cols(symbol_names)
    dg = np.asarray(downstream_grads, dtype=np.float32)
    out = np.zeros((len(parsed), len(symbol_names)), dtype=np.complex128)
    for i, (n, index, items) in enumerate(parsed):
        gates = [g for _, g in items]
        if not gates:
            continue
        psi = simulate(gates, n)
        chi = np.zeros_like(psi)
        for j in range(others.shape[1]):
            om = decode_program(others[i, j])
            og = [build_gate(op, index, {}) for mom in om for op in mom]
            phi = simulate(og, n) if og else np.eye(1, 2 ** n, dtype=np.complex128)[0].reshape(psi.shape)
            chi = chi + float(dg[i, j]) * phi
        for g in reversed(gates):
            mdag = np.conj(g.matrix.T)
            psi = apply_matrix(psi, n, mdag, g.qubits, g.controls, g.cvals)
            for sym, dm in g.grads:
                phi = psi
                if g.controls:
                    mask = np.zeros([2] * n, dtype=bool)
                    sl = [slice(None)] * n
                    for c, v in zip(g.controls, g.cvals):
                        sl[c] = int(v)
                    mask[tuple(sl)] = True
                    phi = np.where(mask, psi, 0)
                phi = apply_matrix(phi, n, dm, g.qubits)
                out[i, cols[sym]] += np.vdot(phi, chi)
            chi = apply_matrix(chi, n, mdag, g.qubits, g.controls, g.cvals)
    return out


def final_probabilities(programs, symbol_names, symbol_values):
    """|psi|^2 per circuit (for statistical checks of the sampler)."""
    parsed, _ = _parse_all(programs, symbol_names, symbol_values)
    res = []
    for n, index, items in parsed:
        if n == 0:
            res.append((0, np.ones(1)))
            continue
        psi = simulate([g for _, g in items], n).reshape(-1)
        res.append((n, np.abs(psi) ** 2))
    return res


def sample_bits_layout(index_samples, n, maxn):
    """tfq_simulate_samples_op.cc:226-243: bit k of the sample (qsim qubit k)
    goes to column maxn-k-1; leading maxn-n columns are -2."""
    s = np.asarray(index_samples, dtype=np.int64)
    out = np.full((len(s), maxn), -2, dtype=np.int8)
    for k in range(n):
        out[:, maxn - k - 1] = (s >> k) & 1
    return out


def adj_grad(programs, symbol_names, symbol_values, pauli_sums,
             downstream_grads, grad_rule="fd"):
    """tfq_adj_grad_op.cc ComputeSmall (:173-284) restated in complex128."""
    parsed, psums = _parse_all(programs, symbol_names, symbol_values,
                               pauli_sums, grad_rule)
    cols = _name_cols(symbol_names)
    dg = np.asarray(downstream_grads, dtype=np.float32)
    out = np.zeros((len(parsed), len(symbol_names)), dtype=np.float64)
    for i, (n, index, items) in enumerate(parsed):
        gates = [g for _, g in items]
        if not gates:
            continue
        psi = simulate(gates, n)
        # AccumulateOperators (util_qsim.h:362-414)
        lam = np.zeros_like(psi)
        for j, terms in enumerate(psums[i]):
            for t in terms:
                lead = F32(dg[i, j] * t["re"])
                if abs(float(lead)) < 1e-5:
                    continue
                if not t["paulis"]:
                    lam = lam + float(lead) * psi
                else:
                    lam = lam + float(lead) * apply_pauli_term(psi, n, t["paulis"], index)
        for g in reversed(gates):
            mdag = np.conj(g.matrix.T)
            psi = apply_matrix(psi, n, mdag, g.qubits, g.controls, g.cvals)
            for sym, dm in g.grads:
                phi = psi
                if g.controls:
                    # zero amplitudes whose controls do not match
                    mask = np.zeros([2] * n, dtype=bool)
                    sl = [slice(None)] * n
                    for c, v in zip(g.controls, g.cvals):
                        sl[c] = int(v)
                    mask[tuple(sl)] = True
                    phi = np.where(mask, psi, 0)
                phi = apply_matrix(phi, n, dm, g.qubits)
                out[i, cols[sym]] += 2.0 * float(np.real(np.vdot(phi, lam)))
            lam = apply_matrix(lam, n, mdag, g.qubits, g.controls, g.cvals)
    return out


# ---------------------------------------------------------------------------
# noisy expectation: exact density matrix
# ---------------------------------------------------------------------------

def _dm_apply(rho, n, m, qubits, controls=(), cvals=()):
    """rho -> M rho M^dagger with rho shaped [2]*(2n) (row axes first)."""
    if controls:
        # build the full controlled unitary on controls+targets
        k = len(qubits)
        c = len(controls)
        dim = 2 ** (c + k)
        full = np.eye(dim, dtype=np.complex128)
        cidx = 0
        for v in cvals:
            cidx = (cidx << 1) | int(v)
        lo = cidx * 2 ** k
        full[lo:lo + 2 ** k, lo:lo + 2 ** k] = m
        m = full
        qubits = list(controls) + list(qubits)
    rho = apply_matrix(rho, 2 * n, m, list(qubits))
    return apply_matrix(rho, 2 * n, np.conj(m), [q + n for q in qubits])


def _final_dm(n, items):
    """Exact density matrix [2^n, 2^n] after the gates and channels."""
    rho = np.zeros([2] * (2 * n), dtype=np.complex128)
    rho[(0,) * (2 * n)] = 1.0
    for it in items:
        if it[0] == "gate":
            g = it[1]
            rho = _dm_apply(rho, n, g.matrix, g.qubits, g.controls, g.cvals)
        else:
            kraus, qs = it[1], it[2]
            acc = 0
            for K in kraus:
                acc = acc + _dm_apply(rho, n, np.asarray(K, dtype=np.complex128), qs)
            rho = acc
    return rho.reshape(2 ** n, 2 ** n)


def noisy_probabilities(programs, symbol_names, symbol_values):
    """(n, measurement probabilities) per noisy circuit: the diagonal of the
    exact density matrix (what tfq_noisy_samples' trajectories sample)."""
    parsed, _ = _parse_all(programs, symbol_names, symbol_values, noisy=True)
    return [(n, np.real(np.diag(_final_dm(n, items))) if items else np.ones(1))
            for n, index, items in parsed]


def noisy_expectation_exact(programs, symbol_names, symbol_values, pauli_sums):
    parsed, psums = _parse_all(programs, symbol_names, symbol_values,
                               pauli_sums, noisy=True)
    n_ops = np.asarray(pauli_sums, dtype=object).shape[1]
    out = np.zeros((len(parsed), n_ops))
    for i, (n, index, items) in enumerate(parsed):
        if not items:
            out[i, :] = -2.0
            continue
        R = _final_dm(n, items)
        for j in range(n_ops):
            v = 0.0
            for t in psums[i][j]:
                if not t["paulis"]:
                    v += float(t["re"])
                    continue
                P = np.ones((1, 1), dtype=np.complex128)
                ops = {index[q]: _PAULI[p] for q, p in t["paulis"]}
                for q in range(n):
                    P = np.kron(P, ops.get(q, _I2))
                v += float(t["re"]) * float(np.real(np.trace(P @ R)))
            out[i, j] = v
    return out
