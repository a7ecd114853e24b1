"""Large-size oracle runs (TEST INFRASTRUCTURE): the complex128 functions of
tfq_oracle.py -- final state, exact density matrix, Pauli-sum expectation --
with the matrix application moved into sv128.c, so that 20-30 qubit states
and 14-qubit density matrices (2^28 entries, 4 GiB) finish in seconds to a
minute on the host cores.

Gate and channel construction, qubit resolution and expectation semantics
are tfq_oracle.py's (which cites the reference for each); only the loops
over amplitudes run in C.  Index convention as there: bit n-1-q of a state
index is resolved qubit q; a density matrix is stored row-major, so its flat
index is row * 2^n + col."""

import ctypes

import numpy as np

from . import build_cpu
from . import tfq_oracle as O

_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_cpu.build_one("sv128"))
        _lib.sv128_apply.restype = ctypes.c_int
        _lib.sv128_apply.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                                     ctypes.c_uint64]
        _lib.sv128_vdot.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                    ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double)]
        _lib.sv128_num_threads.restype = ctypes.c_int
    return _lib


def num_threads():
    return _load().sv128_num_threads()


def _apply(vec, nbits, m, bits, cmask=0, cval=0):
    m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    b = np.ascontiguousarray(np.asarray(bits, dtype=np.int32))
    rc = _load().sv128_apply(vec.ctypes.data, nbits, m.ctypes.data, len(bits),
                             b.ctypes.data, cmask, cval)
    if rc != 0:
        raise ValueError("sv128_apply rejected its arguments")


def _ctrl(n, controls, cvals, shift=0):
    mask = val = 0
    for c, v in zip(controls, cvals):
        mask |= 1 << (n - 1 - c + shift)
        val |= (int(v) & 1) << (n - 1 - c + shift)
    return mask, val


def final_state(n, gates):
    """tfq_oracle.simulate, flat complex128 [2^n]."""
    psi = np.zeros(2 ** n, dtype=np.complex128)
    psi[0] = 1.0
    for g in gates:
        cm, cv = _ctrl(n, g.controls, g.cvals)
        _apply(psi, n, g.matrix, [n - 1 - q for q in g.qubits], cm, cv)
    return psi


def simulate_state_row(program, symbol_names, symbol_values_row):
    """The final state of one program (tfq_oracle.simulate_state's row)."""
    parsed, _ = O._parse_all([program], symbol_names,
                             np.asarray(symbol_values_row, np.float32)[None, :])
    n, index, items = parsed[0]
    return n, index, final_state(n, [g for _, g in items])


def _apply_pauli(psi, n, paulis, index):
    out = psi.copy()
    for qid, p in paulis:
        _apply(out, n, O._PAULI[p], [n - 1 - index[qid]])
    return out


def expectation(psi, n, terms, index):
    """ComputeExpectationQsim semantics (as tfq_oracle.expectation)."""
    v = 0.0
    re, im = ctypes.c_double(), ctypes.c_double()
    for t in terms:
        if not t["paulis"]:
            v += float(t["re"])
            continue
        phi = _apply_pauli(psi, n, t["paulis"], index)
        _load().sv128_vdot(psi.ctypes.data, phi.ctypes.data, psi.size, ctypes.byref(re),
                           ctypes.byref(im))
        v += float(t["re"]) * re.value
    return v


def simulate_expectation_row(program, symbol_names, symbol_values_row, pauli_sums_row):
    parsed, psums = O._parse_all([program], symbol_names,
                                 np.asarray(symbol_values_row, np.float32)[None, :],
                                 [list(pauli_sums_row)])
    n, index, items = parsed[0]
    if not items:
        return np.full(len(pauli_sums_row), -2.0)
    psi = final_state(n, [g for _, g in items])
    return np.array([expectation(psi, n, terms, index) for terms in psums[0]])


# -- density matrices ---------------------------------------------------------

def _superop(kraus):
    """sum_k K (x) conj(K): the map rho -> sum_k K rho K^dag on the bit pair
    (row bit, column bit) of one qubit, row bit the more significant."""
    return sum(np.kron(np.asarray(K, np.complex128), np.conj(np.asarray(K, np.complex128)))
               for K in kraus)


def final_dm(n, items):
    """tfq_oracle._final_dm as a flat row-major complex128 [4^n].

    Consecutive operations on one qubit alone (uncontrolled one-qubit gates
    and the one-qubit channels) are composed first, as complex128 4 x 4
    superoperators; anything on more qubits, or with controls, flushes the
    pending maps of the qubits it touches, then applies M to the row bits
    and conj(M) to the column bits."""
    rho = np.zeros(4 ** n, dtype=np.complex128)
    rho[0] = 1.0
    pend = {}

    def flush(q):
        S = pend.pop(q, None)
        if S is not None:
            _apply(rho, 2 * n, S, [2 * n - 1 - q, n - 1 - q])

    for it in items:
        if it[0] == "gate":
            g = it[1]
            if len(g.qubits) == 1 and not g.controls:
                q = g.qubits[0]
                S = _superop([g.matrix])
                pend[q] = S @ pend[q] if q in pend else S
                continue
            for q in list(g.qubits) + list(g.controls):
                flush(q)
            cm, cv = _ctrl(n, g.controls, g.cvals, shift=n)
            _apply(rho, 2 * n, g.matrix, [2 * n - 1 - q for q in g.qubits], cm, cv)
            cm, cv = _ctrl(n, g.controls, g.cvals)
            _apply(rho, 2 * n, np.conj(g.matrix), [n - 1 - q for q in g.qubits], cm, cv)
        else:
            kraus, qs = it[1], it[2]
            if len(qs) != 1:
                raise ValueError("multi-qubit channels are not part of the gate set")
            q = qs[0]
            S = _superop(kraus)
            pend[q] = S @ pend[q] if q in pend else S
    for q in list(pend):
        flush(q)
    return rho


def pauli_trace(rho, n, paulis, index):
    """Tr(P rho) for a Pauli string P: sum_c <c xor x| P |c> rho[c, c xor x]."""
    dim = 2 ** n
    c = np.arange(dim, dtype=np.int64)
    x = 0
    phase = np.ones(dim, dtype=np.complex128)
    for qid, p in paulis:
        b = n - 1 - index[qid]
        bit = (c >> b) & 1
        if p in ("X", "Y"):
            x |= 1 << b
        if p == "Z":
            phase *= np.where(bit == 1, -1.0, 1.0)
        elif p == "Y":  # Y|0> = i|1>, Y|1> = -i|0>
            phase *= np.where(bit == 1, -1j, 1j)
    r = c ^ x
    return float(np.real(np.sum(phase * rho.reshape(dim, dim)[c, r])))


def noisy_expectation_exact(programs, symbol_names, symbol_values, pauli_sums):
    """tfq_oracle.noisy_expectation_exact through final_dm."""
    parsed, psums = O._parse_all(programs, symbol_names, symbol_values, pauli_sums,
                                 noisy=True)
    n_ops = np.asarray(pauli_sums, dtype=object).shape[1]
    out = np.zeros((len(parsed), n_ops))
    for i, (n, index, items) in enumerate(parsed):
        if not items:
            out[i, :] = -2.0
            continue
        rho = final_dm(n, items)
        for j in range(n_ops):
            v = 0.0
            for t in psums[i][j]:
                if not t["paulis"]:
                    v += float(t["re"])
                else:
                    v += float(t["re"]) * pauli_trace(rho, n, t["paulis"], index)
            out[i, j] = v
        del rho
    return out
