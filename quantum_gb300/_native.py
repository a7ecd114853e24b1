"""ctypes binding of the C ABI in include/tfq_gb300.h.

The library is the in-tree build product quantum_gb300/_lib/libtfq_gb300.so
(`python -m quantum_gb300.build`).  There is no fallback: if the library is
missing every op raises.
"""

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

c_char_pp = ctypes.POINTER(ctypes.c_char_p)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_void_p = ctypes.c_void_p


class NativeLibraryMissing(RuntimeError):
    pass


class InvalidArgumentError(ValueError):
    """tensorflow.errors.InvalidArgumentError counterpart."""


class ResourceExhaustedError(MemoryError):
    """tensorflow.errors.ResourceExhaustedError counterpart."""


class UnimplementedError(NotImplementedError):
    pass


class InternalError(RuntimeError):
    pass


_ERRORS = {3: InvalidArgumentError, 8: ResourceExhaustedError,
           12: UnimplementedError, 13: InternalError}

EXPORTED = (
    "tfqg_last_error", "tfqg_version", "tfqg_batch_create",
    "tfqg_batch_max_num_qubits", "tfqg_batch_destroy",
    "tfqg_batch_expectation", "tfqg_batch_state", "tfqg_batch_samples",
    "tfqg_batch_adj_grad", "tfqg_batch_noisy_expectation",
    "tfqg_simulate_expectation", "tfqg_adj_grad", "tfqg_noisy_expectation",
    "tfqg_batch_sampled_expectation", "tfqg_simulate_sampled_expectation",
    "tfqg_batch_create_inner_product", "tfqg_batch_inner_product", "tfqg_inner_product",
    "tfqg_batch_inner_product_grad", "tfqg_batch_noisy_sampled_expectation",
    "tfqg_batch_noisy_samples", "tfqg_noisy_sampled_expectation", "tfqg_noisy_samples",
    "tfqg_release_cached_memory",
)


def _declare(lib):
    lib.tfqg_last_error.restype = ctypes.c_char_p
    lib.tfqg_version.restype = ctypes.c_char_p
    lib.tfqg_batch_graph_create.argtypes = [c_void_p, ctypes.c_int, c_void_p, ctypes.c_int32,
                                            ctypes.c_uint64, c_void_p, c_void_p,
                                            ctypes.POINTER(c_void_p)]
    lib.tfqg_graph_launch.argtypes = [c_void_p, c_void_p]
    lib.tfqg_graph_destroy.argtypes = [c_void_p]
    lib.tfqg_graph_destroy.restype = None
    lib.tfqg_batch_create.argtypes = [
        c_char_pp, c_int64_p, ctypes.c_int64, c_char_pp, c_int64_p,
        ctypes.c_int64, c_char_pp, c_int64_p, ctypes.c_int64, ctypes.c_int,
        ctypes.POINTER(c_void_p)]
    lib.tfqg_batch_max_num_qubits.argtypes = [c_void_p,
                                              ctypes.POINTER(ctypes.c_int32)]
    lib.tfqg_batch_destroy.argtypes = [c_void_p]
    lib.tfqg_batch_destroy.restype = None
    lib.tfqg_batch_expectation.argtypes = [c_void_p, c_void_p, c_void_p,
                                           ctypes.c_int, c_void_p]
    lib.tfqg_batch_state.argtypes = [c_void_p, c_void_p, c_void_p,
                                     ctypes.c_int, c_void_p]
    lib.tfqg_batch_samples.argtypes = [c_void_p, c_void_p, ctypes.c_int32,
                                       ctypes.c_uint64, c_void_p, ctypes.c_int,
                                       c_void_p]
    lib.tfqg_batch_adj_grad.argtypes = [c_void_p, c_void_p, c_void_p,
                                        ctypes.c_int, c_void_p, ctypes.c_int,
                                        c_void_p]
    lib.tfqg_batch_expectation_noalloc.argtypes = [c_void_p, c_void_p, c_void_p,
                                                   c_void_p]
    lib.tfqg_batch_noisy_expectation.argtypes = [
        c_void_p, c_void_p, c_void_p, ctypes.c_uint64, c_void_p, ctypes.c_int,
        c_void_p]
    lib.tfqg_batch_create_inner_product.argtypes = [
        c_char_pp, c_int64_p, ctypes.c_int64, c_char_pp, c_int64_p, ctypes.c_int64,
        c_char_pp, c_int64_p, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(c_void_p)]
    lib.tfqg_batch_inner_product.argtypes = [c_void_p, c_void_p, c_void_p, ctypes.c_int,
                                             c_void_p]
    lib.tfqg_batch_inner_product_grad.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p,
                                                  ctypes.c_int, c_void_p]
    lib.tfqg_batch_noisy_sampled_expectation.argtypes = [
        c_void_p, c_void_p, c_void_p, ctypes.c_uint64, c_void_p, ctypes.c_int, c_void_p]
    lib.tfqg_batch_noisy_samples.argtypes = [c_void_p, c_void_p, ctypes.c_int32,
                                             ctypes.c_uint64, c_void_p, ctypes.c_int,
                                             c_void_p]
    lib.tfqg_batch_sampled_expectation.argtypes = [
        c_void_p, c_void_p, c_void_p, ctypes.c_uint64, c_void_p, ctypes.c_int,
        c_void_p]
    for name in ("tfqg_batch_create", "tfqg_batch_max_num_qubits",
                 "tfqg_batch_expectation", "tfqg_batch_state",
                 "tfqg_batch_samples", "tfqg_batch_adj_grad",
                 "tfqg_batch_noisy_expectation", "tfqg_batch_expectation_noalloc",
                 "tfqg_batch_sampled_expectation", "tfqg_simulate_sampled_expectation",
                 "tfqg_batch_create_inner_product", "tfqg_batch_inner_product",
                 "tfqg_inner_product", "tfqg_batch_inner_product_grad",
                 "tfqg_batch_noisy_sampled_expectation", "tfqg_batch_noisy_samples",
                 "tfqg_noisy_sampled_expectation", "tfqg_noisy_samples",
                 "tfqg_simulate_expectation",
                 "tfqg_adj_grad", "tfqg_noisy_expectation"):
        getattr(lib, name).restype = ctypes.c_int


def lib():
    """Load (once) and return the native library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.lib_path()
            if not os.path.exists(path):
                raise NativeLibraryMissing(
                    f"{path} is missing; build it with "
                    "`python -m quantum_gb300.build`")
            handle = ctypes.CDLL(path)
            _declare(handle)
            _lib = handle
    return _lib


def check(rc):
    if rc != 0:
        msg = lib().tfqg_last_error().decode("utf-8", "replace")
        raise _ERRORS.get(rc, InternalError)(msg)


def string_array(items):
    """(char**, int64*, keepalive) for a sequence of bytes/str."""
    bs = [x if isinstance(x, (bytes, bytearray)) else str(x).encode("utf-8")
          for x in items]
    bs = [bytes(x) for x in bs]
    n = len(bs)
    ptrs = (ctypes.c_char_p * max(n, 1))(*bs) if n else (ctypes.c_char_p * 1)()
    lens = (ctypes.c_int64 * max(n, 1))(*[len(x) for x in bs])
    return ctypes.cast(ptrs, c_char_pp), ctypes.cast(lens, c_int64_p), (bs, ptrs, lens)


# -- internal controls (tests and benchmarks) -------------------------------
SIM_MODES = {"expect": 0, "state": 1, "sample": 2, "adjoint": 3, "noisy": 4,
             "wide": 5}


def batch_specialization(handle, mode=None):
    """Run-time specialization state of a batch handle.

    mode: None leaves it unchanged, -1 turns it off, 0 automatic, 1 forced.
    Returns (signatures, active_modes, last_error): active_modes is the set
    of module names ("expect" ... "noisy", "wide" for the wide-row pass)
    whose specialized module is loaded."""
    L = lib()
    f = L.tfqg_internal_batch_jit
    f.argtypes = [c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int32),
                  ctypes.POINTER(ctypes.c_int32), ctypes.c_char_p, ctypes.c_int64]
    f.restype = ctypes.c_int
    nsig, active = ctypes.c_int32(), ctypes.c_int32()
    err = ctypes.create_string_buffer(4096)
    check(f(handle, 2 if mode is None else int(mode), ctypes.byref(nsig),
            ctypes.byref(active), err, 4096))
    modes = {k for k, v in SIM_MODES.items() if active.value >> v & 1}
    return nsig.value, modes, err.value.decode("utf-8", "replace")


def specialization_compile_check(handle, mode):
    """Generate and compile (no load, no GPU) the specialized module of
    `mode` for a batch handle. Raises with the compiler log on failure;
    returns the log (ptxas resource usage) on success."""
    L = lib()
    f = L.tfqg_internal_jit_compile_check
    f.argtypes = [c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int64]
    f.restype = ctypes.c_int
    err = ctypes.create_string_buffer(16384)
    rc = f(handle, SIM_MODES[mode], err, 16384)
    if rc != 0:
        raise _ERRORS.get(rc, InternalError)(err.value.decode("utf-8", "replace"))
    return err.value.decode("utf-8", "replace")


def set_wide_min_qubits(n):
    """Qubit count from which forward-mode rows of batches created from now
    on run as wide rows (the whole grid on one state); returns the previous
    value."""
    f = lib().tfqg_internal_set_wide_min_qubits
    f.argtypes = [ctypes.c_int]
    f.restype = ctypes.c_int
    return f(int(n))


def set_gate_fusion(on):
    """Gate fusion of forward plans on or off for batches created from now
    on; returns the previous setting."""
    f = lib().tfqg_internal_set_gate_fusion
    f.argtypes = [ctypes.c_int]
    f.restype = ctypes.c_int
    return bool(f(1 if on else 0))


def set_tensor_core_gates(mode):
    """Forward passes of wide rows as 5-qubit fused blocks on the tensor
    cores: False / 0 never (tile passes on the FP32 pipe), True / 1 always,
    "auto" / 2 (the default) for rows of 24 qubits and more; for calls made
    from now on.  Returns the previous mode (0, 1 or 2)."""
    f = lib().tfqg_internal_set_tensor_core_gates
    f.argtypes = [ctypes.c_int]
    f.restype = ctypes.c_int
    m = 2 if mode == "auto" else int(mode)
    return int(f(m))


def tc_apply(psi_ptr, n, u_ptr, targets, status_ptr, stream=0, grid=0):
    """One launch of the tensor-core 5-qubit block kernel on device buffers:
    psi (2^n complex64) <- U (32 x 32 complex64, row-major) on the ascending
    bits `targets`; status (device int32) is set to 1 on an MMA wait
    timeout.  Raises on a launch error."""
    f = lib().tfqg_internal_tc_apply
    f.argtypes = [c_void_p, ctypes.c_int, c_void_p, c_void_p, c_void_p, ctypes.c_int,
                  c_void_p]
    f.restype = ctypes.c_int
    tgt = (ctypes.c_int32 * 5)(*[int(t) for t in targets])
    rc = f(psi_ptr, int(n), u_ptr, tgt, status_ptr, int(grid), stream)
    if rc != 0:
        raise RuntimeError(f"tc_apply launch failed: cudaError {rc}")


def tc_sweep(psi_ptr, n, u0_ptr, u1_ptr, targets0, targets1, status_ptr, stream=0, grid=0):
    """One two-block tensor-core sweep on device buffers: psi (2^n complex64)
    <- U1 (targets1) U0 (targets0), 32 x 32 complex64 row-major each;
    status (device int32) is set to 1 on a timed-out wait.  Raises on a
    launch error (including blocks that cannot share a sweep)."""
    f = lib().tfqg_internal_tc_sweep
    f.argtypes = [c_void_p, ctypes.c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                  ctypes.c_int, c_void_p]
    f.restype = ctypes.c_int
    t0 = (ctypes.c_int32 * 5)(*[int(t) for t in targets0])
    t1 = (ctypes.c_int32 * 5)(*[int(t) for t in targets1])
    rc = f(psi_ptr, int(n), u0_ptr, u1_ptr, t0, t1, status_ptr, int(grid), stream)
    if rc != 0:
        raise RuntimeError(f"tc_sweep launch failed: cudaError {rc}")


def tc_grid():
    """CTAs of a tensor-core block launch on the current device."""
    f = lib().tfqg_internal_tc_grid
    f.argtypes = []
    f.restype = ctypes.c_int
    return int(f())


def tc_blocks(handle, k):
    """Tensor-core blocks that the k-th wide row of a batch ran in its last
    forward call (-1: it ran tile passes, or has not run)."""
    f = lib().tfqg_internal_tc_blocks
    f.argtypes = [c_void_p, ctypes.c_int64]
    f.restype = ctypes.c_int
    return int(f(handle, int(k)))


def tc_sweeps(handle, k):
    """State sweeps (kernel launches) of the tensor-core blocks of the k-th
    wide row in its last forward call (-1: it ran tile passes)."""
    f = lib().tfqg_internal_tc_sweeps
    f.argtypes = [c_void_p, ctypes.c_int64]
    f.restype = ctypes.c_int
    return int(f(handle, int(k)))


def set_tc_sweep(on):
    """Two consecutive tensor-core blocks share one state sweep where their
    targets allow it (True) or every block sweeps alone (False, the
    default), for calls made from now on; returns the previous setting."""
    f = lib().tfqg_internal_set_tc_sweep
    f.argtypes = [ctypes.c_int]
    f.restype = ctypes.c_int
    return bool(f(1 if on else 0))


def tc_status(handle):
    """Status word of the batch's tensor-core kernels: 0, or 1 when an MMA
    completion wait timed out (synchronizes the device)."""
    f = lib().tfqg_internal_tc_status
    f.argtypes = [c_void_p]
    f.restype = ctypes.c_int
    return int(f(handle))


def tc_inject_status(status):
    """Test hook: calls made from now on treat the tensor-core status word
    as `status` (nonzero: an MMA completion wait timed out), without a
    timeout on the GPU; 0 restores the real read-back.  A lockstep call
    captured in a graph while the hook is set writes status 1 into the
    device word after its tensor-core launches; `status` 2 does only that
    (ordinary calls read the real word).  Returns the previous setting."""
    f = lib().tfqg_internal_tc_inject_status
    f.argtypes = [ctypes.c_int]
    f.restype = ctypes.c_int
    return int(f(int(status)))


def tc_plan(handle, row, row_values, max_blocks=4096):
    """Host copy of a row's tensor-core block plan: a list of (targets,
    matrix) with the 5 target bits ascending and the 32 x 32 complex128
    product of the member gates (index bit i = targets[i]), or None when the
    row has no plan."""
    import numpy as np
    f = lib().tfqg_internal_tc_plan
    f.argtypes = [c_void_p, ctypes.c_int64, c_void_p, c_void_p, c_void_p,
                  ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    f.restype = ctypes.c_int
    vals = np.ascontiguousarray(row_values, dtype=np.float32)
    tgt = np.zeros((max_blocks, 5), dtype=np.int32)
    mats = np.zeros((max_blocks, 32, 32, 2), dtype=np.float64)
    count = ctypes.c_int64(0)
    rc = f(handle, int(row), vals.ctypes.data if vals.size else None,
           tgt.ctypes.data, mats.ctypes.data, max_blocks, ctypes.byref(count))
    if rc != 0:
        raise _ERRORS.get(rc, InternalError)("tc_plan failed")
    if count.value < 0:
        return None
    assert count.value <= max_blocks
    m = mats[:count.value, ..., 0] + 1j * mats[:count.value, ..., 1]
    return [(tuple(int(x) for x in tgt[i]), m[i]) for i in range(count.value)]


def forward_plan_gates(handle, row, row_values):
    """The gates of a row's forward plan in execution order, with matrices
    bound on the host: a list of (nq, b0, b1, cmask, cval, kind, matrix)."""
    import numpy as np
    f = lib().tfqg_internal_forward_plan_gates
    f.argtypes = [c_void_p, ctypes.c_int64, c_void_p, c_void_p, c_void_p,
                  ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    f.restype = ctypes.c_int
    vals = np.ascontiguousarray(row_values, dtype=np.float32)
    if vals.size == 0:
        vals = np.zeros(1, np.float32)
    count = ctypes.c_int64()
    check(f(handle, int(row), vals.ctypes.data, None, None, 0, ctypes.byref(count)))
    k = count.value
    meta = np.zeros((max(k, 1), 6), np.int32)
    mats = np.zeros((max(k, 1), 32), np.float32)
    check(f(handle, int(row), vals.ctypes.data, meta.ctypes.data,
            mats.ctypes.data, k, ctypes.byref(count)))
    out = []
    for i in range(k):
        nq = int(meta[i, 0])
        m = (mats[i, 0::2] + 1j * mats[i, 1::2]).astype(np.complex128)
        m = m[:4].reshape(2, 2) if nq == 1 else m.reshape(4, 4)
        out.append((nq, int(meta[i, 1]), int(meta[i, 2]),
                    int(meta[i, 3]) & 0xFFFFFFFF, int(meta[i, 4]) & 0xFFFFFFFF,
                    int(meta[i, 5]), m))
    return out


def program_cache(on=None):
    """Compiled-program cache: on=True/False switches it (False also empties
    it), None leaves it. Returns (enabled before the call, hits, misses)."""
    f = lib().tfqg_internal_program_cache
    f.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    f.restype = ctypes.c_int
    h, m = ctypes.c_int64(), ctypes.c_int64()
    prev = f(-1 if on is None else int(bool(on)), ctypes.byref(h), ctypes.byref(m))
    return bool(prev), h.value, m.value


def program_cache_capacity(nbytes=0):
    """Capacity of the compiled-program cache in bytes (0 leaves it; the
    default is TFQG_PROGRAM_CACHE_BYTES, else 1 GiB); returns the previous
    capacity."""
    f = lib().tfqg_internal_program_cache_bytes
    f.argtypes = [ctypes.c_int64]
    f.restype = ctypes.c_int64
    return int(f(int(nbytes)))


def program_cache_size():
    """(entries, bytes) held by the compiled-program cache."""
    f = lib().tfqg_internal_program_cache_size
    f.argtypes = [ctypes.POINTER(ctypes.c_int64)]
    f.restype = ctypes.c_int64
    nb = ctypes.c_int64()
    n = f(ctypes.byref(nb))
    return int(n), nb.value


def batch_fingerprint(handle):
    """FNV-1a hash of a batch's packed host tables."""
    f = lib().tfqg_internal_batch_fingerprint
    f.argtypes = [c_void_p]
    f.restype = ctypes.c_uint64
    return int(f(handle))


def row_sweeps(handle, row):
    """(forward passes, measurement passes) of a row's plan: each forward
    pass reads and writes the state once, each measurement pass reads it."""
    f = lib().tfqg_internal_row_sweeps
    f.argtypes = [c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32),
                  ctypes.POINTER(ctypes.c_int32)]
    f.restype = ctypes.c_int
    a, m = ctypes.c_int32(), ctypes.c_int32()
    check(f(handle, int(row), ctypes.byref(a), ctypes.byref(m)))
    return a.value, m.value


def set_lock_min_qubits(n):
    """Qubit count from which streamed rows (not wide) of batches created
    from now on run in lockstep over the whole grid in the forward modes;
    above 21 turns lockstep off.  Returns the previous value."""
    f = lib().tfqg_internal_set_lock_min_qubits
    f.argtypes = [ctypes.c_int]
    f.restype = ctypes.c_int
    return int(f(int(n)))


def set_lock_arena_amps(amps):
    """Largest lockstep group (amplitudes of its rows' states together) for
    batches created from now on; returns the previous value."""
    f = lib().tfqg_internal_set_lock_arena_amps
    f.argtypes = [ctypes.c_int64]
    f.restype = ctypes.c_int64
    return int(f(int(amps)))


def batch_lock_rows(handle):
    """(lockstep rows, lockstep groups) of a batch."""
    f = lib().tfqg_internal_batch_lock_rows
    f.argtypes = [c_void_p]
    f.restype = ctypes.c_int
    g = lib().tfqg_internal_batch_lock_groups
    g.argtypes = [c_void_p]
    g.restype = ctypes.c_int
    return int(f(handle)), int(g(handle))


def set_lock_tc(mode):
    """Lockstep rows of batches created from now on run their gates as
    5-qubit tensor-core blocks (1 or True), as tile passes (0 or False), or
    as blocks from 15 qubits (2, the default), unless a per-qubit-count
    policy says otherwise.  Returns the previous setting."""
    f = lib().tfqg_internal_set_lock_tc
    f.argtypes = [ctypes.c_int]
    f.restype = ctypes.c_int
    return int(f(int(mode)))


def set_tc_lock_persistent(on):
    """Lockstep tensor-core rows of later calls run as one persistent launch
    per lockstep group (True, the default: CTAs take units from a queue,
    each waiting for its row's earlier blocks) or as one launch per block
    index and variant (False).  Returns the previous setting."""
    f = lib().tfqg_internal_set_tc_lock_persistent
    f.argtypes = [ctypes.c_int]
    f.restype = ctypes.c_int
    return bool(f(1 if on else 0))


def batch_lock_punits(handle):
    """The persistent form's units of a batch in queue order: an int64
    array of rows (group, row slot, batch row, need, first chunk, chunks)."""
    import numpy as np
    f = lib().tfqg_internal_batch_lock_punits
    f.argtypes = [c_void_p, c_void_p, ctypes.c_int64]
    f.restype = ctypes.c_int64
    n = f(handle, None, 0)
    out = np.zeros((max(n, 1), 6), np.int64)
    f(handle, out.ctypes.data, n)
    return out[:n]


def batch_lock_tc(handle):
    """(tensor-core blocks, kernel units) of a batch's lockstep rows."""
    f = lib().tfqg_internal_batch_lock_tc
    f.argtypes = [c_void_p, ctypes.POINTER(ctypes.c_int64)]
    f.restype = ctypes.c_int64
    u = ctypes.c_int64()
    nb = f(handle, ctypes.byref(u))
    return int(nb), u.value


def set_wide_few_rows(rows):
    """Batches that stream fewer than `rows` rows run their rows of 17+
    qubits as wide rows (0: never); for batches created from now on.
    Returns the previous value."""
    f = lib().tfqg_internal_set_wide_few_rows
    f.argtypes = [ctypes.c_int]
    f.restype = ctypes.c_int
    return f(int(rows))


def batch_wide_rows(handle):
    f = lib().tfqg_internal_batch_wide_rows
    f.argtypes = [c_void_p]
    f.restype = ctypes.c_int
    return f(handle)
