"""The reference's op API on the GB300 kernels.

Same names, argument order and meaning as
tensorflow_quantum/core/ops/tfq_simulate_ops.py:22-135 (tfq_simulate_expectation,
tfq_simulate_state, tfq_simulate_samples),
tensorflow_quantum/core/ops/tfq_adj_grad_op.py:22-48 (tfq_adj_grad) and
tensorflow_quantum/core/ops/noise/noisy_expectation_op.py:23-98
(noise.expectation).  Inputs may be numpy arrays / Python lists (results are
numpy arrays) or torch tensors (results are torch tensors on the device of
`symbol_values`; CUDA tensors run asynchronously on the current stream).

Shape errors raise InvalidArgumentError with the reference's messages
(parse_context.cc); parse and resolution errors come from the native library.
"""

import ctypes
import os

import numpy as np

from . import _native
from ._native import InvalidArgumentError  # noqa: F401  (re-export)

KIND_FORWARD, KIND_ADJOINT, KIND_NOISY, KIND_INNER = 0, 1, 2, 3
GRAD_REFERENCE_FD, GRAD_EXACT = 0, 1

try:  # torch is optional for the numpy path
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_torch(x):
    return torch is not None and isinstance(x, torch.Tensor)


def _strings(x, name, rank):
    """Flatten a (possibly nested) string tensor of the given rank."""
    if _is_torch(x):
        raise InvalidArgumentError(f"{name} must be a string tensor")
    arr = np.asarray(x, dtype=object)
    if arr.ndim != rank:
        raise InvalidArgumentError(
            f"{name} must be rank {rank}. Got rank {arr.ndim}.")
    flat = [v if isinstance(v, (bytes, bytearray)) else
            (v.encode("utf-8") if isinstance(v, str) else bytes(v))
            for v in arr.reshape(-1)]
    return flat, arr.shape


def _values(symbol_values):
    """symbol_values as float32 (numpy, or contiguous torch tensor)."""
    if _is_torch(symbol_values):
        v = symbol_values.detach()
        if v.dim() != 2:
            raise InvalidArgumentError(
                f"symbol_values must be rank 2. Got rank {v.dim()}.")
        return v.to(torch.float32).contiguous()
    v = np.asarray(symbol_values, dtype=np.float32)
    if v.ndim == 1 and v.size == 0:
        v = v.reshape(0, 0)
    if v.ndim != 2:
        raise InvalidArgumentError(
            f"symbol_values must be rank 2. Got rank {v.ndim}.")
    return np.ascontiguousarray(v)


def _ptr(x):
    if _is_torch(x):
        return ctypes.c_void_p(x.data_ptr())
    return x.ctypes.data_as(ctypes.c_void_p)


def _stream(x):
    if _is_torch(x) and x.is_cuda:
        return ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
    return ctypes.c_void_p(0)


class Batch:
    """A compiled batch: programs (+ pauli sums) parsed, resolved and planned
    once; run many times with new symbol values.  This is the handle the TF
    op shim and the torch autograd function hold."""

    def __init__(self, programs, symbol_names, pauli_sums=None,
                 kind=KIND_FORWARD):
        progs, pshape = _strings(programs, "programs", 1)
        names, _ = _strings(symbol_names, "symbol_names", 1)
        if pauli_sums is not None:
            ps, psshape = _strings(pauli_sums, "pauli_sums", 2)
            if psshape[0] != pshape[0]:
                raise InvalidArgumentError(
                    "Number of circuits and PauliSums do not match. Got "
                    f"{pshape[0]} circuits and {psshape[0]} paulisums.")
            n_ops = psshape[1]
        else:
            ps, n_ops = [], 0
        self.batch_size = pshape[0]
        self.num_symbols = len(names)
        self.num_ops = n_ops
        self.kind = kind
        lib = _native.lib()
        pp, pl, k1 = _native.string_array(progs)
        npp, npl, k2 = _native.string_array(names)
        spp, spl, k3 = _native.string_array(ps)
        h = ctypes.c_void_p()
        _native.check(lib.tfqg_batch_create(
            pp, pl, self.batch_size, npp, npl, self.num_symbols,
            spp if pauli_sums is not None else None, spl, n_ops, kind,
            ctypes.byref(h)))
        self._h = h
        mq = ctypes.c_int32()
        _native.check(lib.tfqg_batch_max_num_qubits(h, ctypes.byref(mq)))
        self.max_num_qubits = mq.value
        del k1, k2, k3

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().tfqg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- helpers ------------------------------------------------------------
    def _check_values(self, v):
        rows, cols = (tuple(v.shape) if _is_torch(v) else v.shape)
        if cols != self.num_symbols:
            raise InvalidArgumentError(
                "Input symbol names and value sizes do not match.")
        if rows != self.batch_size:
            raise InvalidArgumentError(
                "Number of circuits and symbol_values do not match. Got "
                f"{self.batch_size} circuits and {rows} symbol values.")

    def _out(self, v, shape, np_dtype, torch_dtype):
        if _is_torch(v):
            return torch.empty(shape, dtype=torch_dtype, device=v.device)
        return np.empty(shape, dtype=np_dtype)

    @staticmethod
    def _device_flag(v):
        return 1 if (_is_torch(v) and v.is_cuda) else 0

    def _host_or_cuda(self, v):
        if _is_torch(v) and not v.is_cuda:
            return v.numpy()
        return v

    # -- ops ----------------------------------------------------------------
    def expectation(self, symbol_values):
        v = self._host_or_cuda(_values(symbol_values))
        self._check_values(v)
        out = self._out(v, (self.batch_size, self.num_ops), np.float32,
                        getattr(torch, "float32", None))
        _native.check(_native.lib().tfqg_batch_expectation(
            self._h, _ptr(v), _ptr(out), self._device_flag(v), _stream(v)))
        return self._wrap(symbol_values, out)

    def state(self, symbol_values):
        v = self._host_or_cuda(_values(symbol_values))
        self._check_values(v)
        out = self._out(v, (self.batch_size, 2 ** self.max_num_qubits),
                        np.complex64, getattr(torch, "complex64", None))
        _native.check(_native.lib().tfqg_batch_state(
            self._h, _ptr(v), _ptr(out), self._device_flag(v), _stream(v)))
        return self._wrap(symbol_values, out)

    def samples(self, symbol_values, num_samples, seed=None):
        v = self._host_or_cuda(_values(symbol_values))
        self._check_values(v)
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        out = self._out(v, (self.batch_size, int(num_samples),
                            self.max_num_qubits), np.int8,
                        getattr(torch, "int8", None))
        _native.check(_native.lib().tfqg_batch_samples(
            self._h, _ptr(v), int(num_samples), seed & (2 ** 64 - 1),
            _ptr(out), self._device_flag(v), _stream(v)))
        return self._wrap(symbol_values, out)

    def adj_grad(self, symbol_values, downstream_grads,
                 grad_rule=GRAD_REFERENCE_FD):
        v = self._host_or_cuda(_values(symbol_values))
        self._check_values(v)
        if _is_torch(v):
            g = downstream_grads
            if not _is_torch(g):
                g = torch.as_tensor(np.asarray(g, dtype=np.float32))
            g = g.detach().to(device=v.device, dtype=torch.float32).contiguous()
            gshape = tuple(g.shape)
        else:
            g = np.ascontiguousarray(np.asarray(
                downstream_grads.cpu().numpy() if _is_torch(downstream_grads)
                else downstream_grads, dtype=np.float32))
            gshape = g.shape
        if len(gshape) != 2:
            raise InvalidArgumentError(
                f"downstream_grads must be rank 2. Got rank {len(gshape)}.")
        if gshape[0] != self.batch_size:
            raise InvalidArgumentError(
                "Number of gradients and circuits do not match. Got "
                f"{gshape[0]} gradients and {self.batch_size} circuits.")
        if gshape[1] != self.num_ops:
            raise InvalidArgumentError(
                "Number of gradients and pauli sum dimension do not match. Got "
                f"{gshape[1]} gradient entries and {self.num_ops} paulis per "
                "circuit.")
        out = self._out(v, (self.batch_size, self.num_symbols), np.float32,
                        getattr(torch, "float32", None))
        _native.check(_native.lib().tfqg_batch_adj_grad(
            self._h, _ptr(v), _ptr(g), int(grad_rule), _ptr(out),
            self._device_flag(v), _stream(v)))
        return self._wrap(symbol_values, out)

    def _num_samples_2d(self, num_samples):
        """num_samples [batch, num_ops] int32 with the reference's checks
        (parse_context.cc:349-381 and the ops' dimension checks)."""
        ns = np.asarray(num_samples.cpu().numpy() if _is_torch(num_samples)
                        else num_samples, dtype=np.int32)
        if ns.ndim != 2:
            raise InvalidArgumentError(
                f"num_samples must be rank 2. Got rank {ns.ndim}.")
        if ns.shape[0] != self.batch_size:
            raise InvalidArgumentError(
                "Dimension 0 of num_samples and pauli_sums do not match.Got "
                f"{ns.shape[0]} lists of sample sizes and {self.batch_size} "
                "lists of pauli sums.")
        if ns.shape[1] != self.num_ops:
            raise InvalidArgumentError(
                "Dimension 1 of num_samples and pauli_sums do not match.Got "
                f"{ns.shape[1]} lists of sample sizes and {self.num_ops} "
                "lists of pauli sums.")
        return np.ascontiguousarray(ns)

    def _counts_call(self, fn, symbol_values, num_samples, seed):
        v = self._host_or_cuda(_values(symbol_values))
        self._check_values(v)
        ns = self._num_samples_2d(num_samples)
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        dev = self._device_flag(v)
        nsp = torch.as_tensor(ns, device=v.device) if dev else ns
        out = self._out(v, (self.batch_size, self.num_ops), np.float32,
                        getattr(torch, "float32", None))
        _native.check(fn(self._h, _ptr(v), _ptr(nsp), seed & (2 ** 64 - 1),
                         _ptr(out), dev, _stream(v)))
        return self._wrap(symbol_values, out)

    def noisy_expectation(self, symbol_values, num_samples, seed=None):
        """Trajectory expectations (noise/noisy_expectation_op.py:23-98);
        num_samples [batch, num_ops] trajectories per entry."""
        return self._counts_call(_native.lib().tfqg_batch_noisy_expectation,
                                 symbol_values, num_samples, seed)

    def noisy_sampled_expectation(self, symbol_values, num_samples, seed=None):
        """Trajectory means of once-per-trajectory term measurements
        (noise/noisy_sampled_expectation_op.py); num_samples [batch,
        num_ops] trajectories per entry."""
        return self._counts_call(_native.lib().tfqg_batch_noisy_sampled_expectation,
                                 symbol_values, num_samples, seed)

    def noisy_samples(self, symbol_values, num_samples, seed=None):
        """int8 [batch, num_samples, max_n]: one sample per trajectory
        (noise/noisy_samples_op.py), the samples op's layout."""
        v = self._host_or_cuda(_values(symbol_values))
        self._check_values(v)
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        out = self._out(v, (self.batch_size, int(num_samples), self.max_num_qubits),
                        np.int8, getattr(torch, "int8", None))
        _native.check(_native.lib().tfqg_batch_noisy_samples(
            self._h, _ptr(v), int(num_samples), seed & (2 ** 64 - 1), _ptr(out),
            self._device_flag(v), _stream(v)))
        return self._wrap(symbol_values, out)

    def sampled_expectation(self, symbol_values, num_samples, seed=None):
        """Expectations estimated from measurement samples
        (tfq_simulate_ops.py:101-135); num_samples [batch, num_ops] samples
        per Pauli term."""
        return self._counts_call(_native.lib().tfqg_batch_sampled_expectation,
                                 symbol_values, num_samples, seed)

    def capture(self, what, values, num_samples=0, seed=0, stream=None):
        """A Graph of one forward call ("expectation", "state" or
        "samples") on CUDA `values`; close it before the batch."""
        return Graph(self, what, values, num_samples, seed, stream)

    @staticmethod
    def _wrap(symbol_values, out):
        if _is_torch(symbol_values) and not _is_torch(out):
            return torch.from_numpy(out)
        return out


class Graph:
    """One forward call of a Batch (expectation, state or samples) captured
    in a CUDA graph (tfqg_batch_graph_create): `replay()` relaunches the
    whole batched call -- matrix build, persistent queue kernel, lockstep and
    wide-row launches -- as one graph launch on the capture stream.  The
    graph reads `values` and writes `out` (torch CUDA tensors held here), so
    writing new symbol values into `values` and replaying gives their
    results; samples replay with the captured seed."""

    _WHAT = {"expectation": 0, "state": 1, "samples": 2}

    def __init__(self, batch, what, values, num_samples=0, seed=0, stream=None):
        if not (_is_torch(values) and values.is_cuda):
            raise InvalidArgumentError("a graph captures device buffers: values must be a "
                                       "CUDA tensor")
        batch._check_values(values)
        self.batch = batch
        self.values = values
        self.stream = stream or torch.cuda.Stream(device=values.device)
        if what == "expectation":
            self.out = torch.empty((batch.batch_size, batch.num_ops), dtype=torch.float32,
                                   device=values.device)
        elif what == "state":
            self.out = torch.empty((batch.batch_size, 2 ** batch.max_num_qubits),
                                   dtype=torch.complex64, device=values.device)
        else:
            self.out = torch.empty((batch.batch_size, int(num_samples),
                                    batch.max_num_qubits), dtype=torch.int8,
                                   device=values.device)
        self.stream.wait_stream(torch.cuda.current_stream(values.device))
        h = ctypes.c_void_p()
        _native.check(_native.lib().tfqg_batch_graph_create(
            batch._h, self._WHAT[what], ctypes.c_void_p(values.data_ptr()), int(num_samples),
            int(seed) & (2 ** 64 - 1), ctypes.c_void_p(self.out.data_ptr()),
            ctypes.c_void_p(self.stream.cuda_stream), ctypes.byref(h)))
        self._g = h

    def replay(self):
        """One graph launch on the capture stream (ordered after the current
        stream's work); returns `out`."""
        cur = torch.cuda.current_stream(self.values.device)
        self.stream.wait_stream(cur)
        _native.check(_native.lib().tfqg_graph_launch(
            self._g, ctypes.c_void_p(self.stream.cuda_stream)))
        cur.wait_stream(self.stream)
        return self.out

    def close(self):
        if getattr(self, "_g", None):
            _native.lib().tfqg_graph_destroy(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class InnerProductBatch(Batch):
    """A compiled tfq_inner_product batch: reference programs (with symbols)
    and their paired other_programs [batch, n_others] (no symbols), parsed and
    resolved once (math_ops/tfq_inner_product.cc:48-166)."""

    def __init__(self, programs, symbol_names, other_programs, with_grads=False):
        progs, pshape = _strings(programs, "programs", 1)
        names, _ = _strings(symbol_names, "symbol_names", 1)
        others, oshape = _strings(other_programs, "other_programs", 2)
        if oshape[0] != pshape[0]:
            raise InvalidArgumentError(
                "programs and other_programs batch dimension do not match. Foud: "
                f"{pshape[0]} and {oshape[0]}")
        self.batch_size = pshape[0]
        self.num_symbols = len(names)
        self.num_ops = 0
        self.num_others = oshape[1]
        self.kind = KIND_INNER
        lib = _native.lib()
        pp, pl, k1 = _native.string_array(progs)
        npp, npl, k2 = _native.string_array(names)
        opp, opl, k3 = _native.string_array(others)
        h = ctypes.c_void_p()
        _native.check(lib.tfqg_batch_create_inner_product(
            pp, pl, self.batch_size, npp, npl, self.num_symbols, opp, opl,
            self.num_others, 1 if with_grads else 0, ctypes.byref(h)))
        self._h = h
        mq = ctypes.c_int32()
        _native.check(lib.tfqg_batch_max_num_qubits(h, ctypes.byref(mq)))
        self.max_num_qubits = mq.value
        del k1, k2, k3

    def inner_product(self, symbol_values):
        """complex64 [batch, n_others]: <psi_i(values_i) | phi_ij>."""
        v = self._host_or_cuda(_values(symbol_values))
        self._check_values(v)
        out = self._out(v, (self.batch_size, self.num_others), np.complex64,
                        getattr(torch, "complex64", None))
        _native.check(_native.lib().tfqg_batch_inner_product(
            self._h, _ptr(v), _ptr(out), self._device_flag(v), _stream(v)))
        return self._wrap(symbol_values, out)

    def inner_product_grad(self, symbol_values, prev_grad):
        """TfqInnerProductGrad's output, complex64 [batch, n_symbols]:
        sum_j prev_grad[i, j] d<psi_i|phi_ij>/d symbol (the batch must be
        created with with_grads=True); prev_grad [batch, n_others] real."""
        v = self._host_or_cuda(_values(symbol_values))
        self._check_values(v)
        if _is_torch(v):
            g = prev_grad if _is_torch(prev_grad) else torch.as_tensor(
                np.asarray(prev_grad))
            if g.is_complex():
                g = g.real
            g = g.detach().to(device=v.device, dtype=torch.float32).contiguous()
            gshape = tuple(g.shape)
        else:
            g = np.asarray(prev_grad.cpu().numpy() if _is_torch(prev_grad) else prev_grad)
            g = np.ascontiguousarray(np.real(g).astype(np.float32))
            gshape = g.shape
        if len(gshape) != 2:
            raise InvalidArgumentError(
                f"downstream_grads must be rank 2. Got rank {len(gshape)}.")
        if gshape[0] != self.batch_size:
            raise InvalidArgumentError(
                "Number of gradients and circuits do not match. Got "
                f"{gshape[0]} gradients and {self.batch_size} circuits.")
        if gshape[1] != self.num_others:
            raise InvalidArgumentError(
                "Number of gradients and other_programs do not match. Got "
                f"{gshape[1]} gradient entries and {self.num_others} other programs.")
        out = self._out(v, (self.batch_size, self.num_symbols), np.complex64,
                        getattr(torch, "complex64", None))
        _native.check(_native.lib().tfqg_batch_inner_product_grad(
            self._h, _ptr(v), _ptr(g), _ptr(out), self._device_flag(v), _stream(v)))
        return self._wrap(symbol_values, out)


# ---------------------------------------------------------------------------
# the reference's functional API
# ---------------------------------------------------------------------------

def tfq_simulate_expectation(programs, symbol_names, symbol_values, pauli_sums):
    """tfq_simulate_ops.py:22-45."""
    v = _values(symbol_values)
    b = Batch(programs, symbol_names, pauli_sums, KIND_FORWARD)
    try:
        return b.expectation(v if not _is_torch(symbol_values) else symbol_values)
    finally:
        b.close()


def tfq_simulate_state(programs, symbol_names, symbol_values):
    """tfq_simulate_ops.py:48-69."""
    b = Batch(programs, symbol_names, None, KIND_FORWARD)
    try:
        return b.state(symbol_values)
    finally:
        b.close()


def tfq_simulate_samples(programs, symbol_names, symbol_values, num_samples,
                         seed=None):
    """tfq_simulate_ops.py:72-98; `num_samples` is a 1-element tensor."""
    ns = np.asarray(num_samples.cpu().numpy() if _is_torch(num_samples)
                    else num_samples)
    if ns.ndim != 1:
        raise InvalidArgumentError(
            f"num_samples must be rank 1. Got rank {ns.ndim}.")
    if ns.shape[0] != 1:
        raise InvalidArgumentError(
            f"num_samples must contain 1 element. Got {ns.shape[0]}.")
    b = Batch(programs, symbol_names, None, KIND_FORWARD)
    try:
        return b.samples(symbol_values, int(ns[0]), seed)
    finally:
        b.close()


def tfq_adj_grad(programs, symbol_names, symbol_values, pauli_sums, prev_grad,
                 grad_rule=GRAD_REFERENCE_FD):
    """tfq_adj_grad_op.py:22-48."""
    b = Batch(programs, symbol_names, pauli_sums, KIND_ADJOINT)
    try:
        return b.adj_grad(symbol_values, prev_grad, grad_rule)
    finally:
        b.close()


def tfq_simulate_sampled_expectation(programs, symbol_names, symbol_values,
                                     pauli_sums, num_samples, seed=None):
    """tfq_simulate_ops.py:101-135."""
    b = Batch(programs, symbol_names, pauli_sums, KIND_FORWARD)
    try:
        return b.sampled_expectation(symbol_values, num_samples, seed)
    finally:
        b.close()


def tfq_inner_product(programs, symbol_names, symbol_values, other_programs):
    """math_ops/inner_product_op.py:72-130 (tfq.math.inner_product)."""
    b = InnerProductBatch(programs, symbol_names, other_programs)
    try:
        return b.inner_product(symbol_values)
    finally:
        b.close()


def inner_product_grad(programs, symbol_names, symbol_values, other_programs,
                       prev_grad):
    """math_ops/inner_product_op.py:22-69 (_inner_product_grad): the complex
    conjugate of TfqInnerProductGrad's output, prev_grad cast to float32."""
    b = InnerProductBatch(programs, symbol_names, other_programs, with_grads=True)
    try:
        out = b.inner_product_grad(symbol_values, prev_grad)
        return out.conj() if _is_torch(out) else np.conj(out)
    finally:
        b.close()


def _one_sample_count(num_samples):
    ns = np.asarray(num_samples.cpu().numpy() if _is_torch(num_samples)
                    else num_samples)
    if ns.ndim != 1:
        raise InvalidArgumentError(f"num_samples must be rank 1. Got rank {ns.ndim}.")
    if ns.shape[0] != 1:
        raise InvalidArgumentError(f"num_samples must contain 1 element. Got {ns.shape[0]}.")
    return int(ns[0])


def noisy_samples(programs, symbol_names, symbol_values, num_samples, seed=None):
    """noise/noisy_samples_op.py (tfq.noise.samples); `num_samples` is a
    1-element tensor."""
    n = _one_sample_count(num_samples)
    b = Batch(programs, symbol_names, None, KIND_NOISY)
    try:
        return b.noisy_samples(symbol_values, n, seed)
    finally:
        b.close()


def noisy_sampled_expectation(programs, symbol_names, symbol_values, pauli_sums,
                              num_samples, seed=None):
    """noise/noisy_sampled_expectation_op.py (tfq.noise.sampled_expectation)."""
    b = Batch(programs, symbol_names, pauli_sums, KIND_NOISY)
    try:
        return b.noisy_sampled_expectation(symbol_values, num_samples, seed)
    finally:
        b.close()


def noisy_expectation(programs, symbol_names, symbol_values, pauli_sums,
                      num_samples, seed=None):
    """noise/noisy_expectation_op.py:23-98 (tfq.noise.expectation)."""
    b = Batch(programs, symbol_names, pauli_sums, KIND_NOISY)
    try:
        return b.noisy_expectation(symbol_values, num_samples, seed)
    finally:
        b.close()
