"""Python side of the CPU restatement (TEST INFRASTRUCTURE): flattens a batch
parsed by the oracle (tfq_oracle.py) and runs oracle/cpu_ref.cc's
expectation + adjoint loops (fused forward, fused partial blocks in the
adjoint sweep, vectorized amplitude loops) over host threads."""

import ctypes

import numpy as np

from . import build_cpu
from . import tfq_oracle as O

_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_cpu.build())
        _lib.cpuref_run.restype = ctypes.c_int
        _lib.cpuref_num_threads.restype = ctypes.c_int
    return _lib


def num_threads():
    return _load().cpuref_num_threads()


class Flat:
    """A batch flattened for cpu_ref.cc."""

    def __init__(self, programs, symbol_names, symbol_values, pauli_sums):
        parsed, psums = O._parse_all(programs, symbol_names, symbol_values,
                                     pauli_sums, "fd")
        cols = O._name_cols(symbol_names)
        self.rows = len(parsed)
        self.n_ops = np.asarray(pauli_sums, dtype=object).shape[1]
        self.num_symbols = len(symbol_names)
        n, goff, nq, b0, b1, cm, cv, mats, ng, gc, dm = ([] for _ in range(11))
        toff, top, tco, foff, fbit, ftyp = [0], [], [], [0], [], []
        goff.append(0)
        for i, (nn, index, items) in enumerate(parsed):
            n.append(nn)
            for _, g in items:
                nq.append(len(g.qubits))
                b0.append(nn - 1 - g.qubits[0])
                b1.append(nn - 1 - g.qubits[1] if len(g.qubits) > 1 else 0)
                m = 0
                v = 0
                for c, val in zip(g.controls, g.cvals):
                    m |= 1 << (nn - 1 - c)
                    v |= (int(val) & 1) << (nn - 1 - c)
                cm.append(m)
                cv.append(v)
                mm = np.zeros(16, np.complex64)
                mm[:g.matrix.size] = g.matrix.reshape(-1)
                mats.append(mm.view(np.float32))
                ng.append(len(g.grads))
                gcol = [0, 0]
                dd = np.zeros((2, 16), np.complex64)
                for k, (sym, d) in enumerate(g.grads):
                    gcol[k] = cols[sym]
                    dd[k, :d.size] = d.reshape(-1)
                gc.extend(gcol)
                dm.append(dd.view(np.float32).reshape(-1))
            goff.append(len(nq))
            for j in range(self.n_ops):
                for t in psums[i][j]:
                    top.append(j)
                    tco.append(float(t["re"]))
                    for qid, p in t["paulis"]:
                        fbit.append(nn - 1 - index[qid])
                        ftyp.append(p.encode())
                    foff.append(len(fbit))
            toff.append(len(top))
        i32 = lambda a: np.ascontiguousarray(np.array(a, dtype=np.int32))
        self.a = dict(
            n=i32(n), goff=np.array(goff, np.int64), nq=i32(nq), b0=i32(b0),
            b1=i32(b1), cm=np.array(cm, np.uint32), cv=np.array(cv, np.uint32),
            mats=np.ascontiguousarray(np.concatenate(mats) if mats else np.zeros(32, np.float32)),
            ng=i32(ng), gc=i32(gc),
            dm=np.ascontiguousarray(np.concatenate(dm) if dm else np.zeros(64, np.float32)),
            toff=np.array(toff, np.int64), top=i32(top),
            tco=np.array(tco, np.float32), foff=np.array(foff, np.int64),
            fbit=i32(fbit), ftyp=np.array(ftyp or [b"Z"], dtype="S1"))

    def run(self, downstream_grads, threads=0, expectation=True, adjoint=True):
        """One expectation op and / or one adjoint-gradient op over the
        rows; returns (expectations [rows, n_ops], gradients [rows, P])."""
        lib = _load()
        a = self.a
        dg = np.ascontiguousarray(np.asarray(downstream_grads, np.float32))
        exp = np.zeros((self.rows, self.n_ops), np.float32)
        grad = np.zeros((self.rows, self.num_symbols), np.float32)
        p = lambda x: x.ctypes.data_as(ctypes.c_void_p)
        lib.cpuref_run(
            ctypes.c_int(self.rows), p(a["n"]), p(a["goff"]), p(a["nq"]),
            p(a["b0"]), p(a["b1"]), p(a["cm"]), p(a["cv"]), p(a["mats"]),
            p(a["ng"]), p(a["gc"]), p(a["dm"]), p(a["toff"]), p(a["top"]),
            p(a["tco"]), p(a["foff"]), p(a["fbit"]), p(a["ftyp"]),
            ctypes.c_int(self.n_ops), ctypes.c_int(self.num_symbols), p(dg),
            p(exp), p(grad), ctypes.c_int(threads), ctypes.c_int(int(expectation)),
            ctypes.c_int(int(adjoint)))
        return exp, grad
