"""Autotuner of the row plan per qubit count.

For every qubit count present in a batch it times, on the current GPU, the
candidate plans of the library's rows and installs the fastest one for rows
of that qubit count in batches created afterwards:

- fusion width: gates applied one by one (width 1), the forward fuser's
  folds of one-qubit chains into two-qubit gates (width 2), or 5-qubit
  blocks on the tensor cores (width 5, streamed rows in lockstep only);
- tile schedule of streamed rows of 15-21 qubits that do not run wide: one
  CTA per row through the persistent queue, or lockstep over the whole grid
  (one launch per pass index, or per block index, across all such rows).

(Rows of 24 qubits and more take 5-qubit tensor-core blocks by default; that
choice is the library's and is not tuned here.)

Timings use a sample of the batch's own rows of each qubit count (up to
`rows_per_bucket`), CUDA events around `repeats` calls after one warm-up
call, and the ops the caller names (expectation, and samples when
`samples > 0`).  Results are cached per GPU name, qubit count and op set in
$TFQG_CACHE_DIR/autotune.json (default ~/.cache/tfq_gb300), so later
processes install them without timing (`use_cache=False` re-times).
"""

import ctypes
import json
import os
import time

import numpy as np

from . import _native, ops

LOCK_QUBITS = range(15, 22)


def set_row_policy(n, fuse=-1, lock=-1):
    """Policy for rows of n qubits in batches created from now on: fuse -1
    (library default), 0 off, 1 on; lock -1 (library default), 0 off (the
    queue), 1 lockstep on tile passes, 2 lockstep on tensor-core blocks.
    n < 0 resets every qubit count."""
    f = _native.lib().tfqg_internal_set_row_policy
    f.argtypes = [ctypes.c_int] * 3
    f.restype = ctypes.c_int
    return int(f(int(n), int(fuse), int(lock)))


def reset():
    """Back to the library's defaults for every qubit count."""
    set_row_policy(-1)


def _cache_path():
    d = os.environ.get("TFQG_CACHE_DIR") or os.path.join(
        os.path.expanduser("~"), ".cache", "tfq_gb300")
    return os.path.join(d, "autotune.json")


def _load_cache():
    try:
        return json.load(open(_cache_path()))
    except (OSError, ValueError):
        return {}


def _save_cache(c):
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(c, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def qubit_counts(programs):
    """Resolved qubit count of every program (host only)."""
    f = _native.lib().tfqg_max_num_qubits
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    f.restype = ctypes.c_int
    out = []
    for p in programs:
        pp, pl, keep = _native.string_array([p])
        mq = ctypes.c_int32()
        _native.check(f(pp, pl, 1, ctypes.byref(mq)))
        out.append(mq.value)
    return out


def _candidates(n):
    c = [(0, -1), (1, -1)]
    if n in LOCK_QUBITS:
        # (the fusion flag does not change tensor-core rows: one candidate)
        c = [(f, lk) for f in (0, 1) for lk in (0, 1)] + [(1, 2)]
    return c


def tune(programs, pauli_sums, symbol_names=(), symbol_values=None, samples=0,
         rows_per_bucket=128, repeats=2, use_cache=True):
    """Times the candidate plans of every qubit count among `programs` and
    installs the fastest; returns {n: {"fuse", "lock", "ms", "candidates",
    "rows", "cached"}}."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    gpu = torch.cuda.get_device_name(dev)
    kinds = "expectation" + (f"+samples{int(samples)}" if samples else "")
    cache = _load_cache() if use_cache else {}
    ns = np.array(qubit_counts(programs))
    vals = (np.zeros((len(programs), 0), np.float32) if symbol_values is None
            else np.asarray(symbol_values, np.float32))
    result = {}
    for n in sorted(set(int(x) for x in ns if x > 0)):
        key = f"{gpu}|n={n}|{kinds}"
        if key in cache:
            fuse, lock = cache[key]["fuse"], cache[key]["lock"]
            set_row_policy(n, fuse, lock)
            result[n] = dict(cache[key], cached=True)
            continue
        idx = np.nonzero(ns == n)[0]
        if len(idx) > rows_per_bucket:
            idx = idx[np.linspace(0, len(idx) - 1, rows_per_bucket).astype(int)]
        progs = [programs[i] for i in idx]
        psums = [pauli_sums[i] for i in idx]
        v = torch.tensor(vals[idx], device=dev)
        timed = {}
        for fuse, lock in _candidates(n):
            set_row_policy(n, fuse, lock)
            b = ops.Batch(progs, list(symbol_names), psums, ops.KIND_FORWARD)

            def call():
                b.expectation(v)
                if samples:
                    b.samples(v, int(samples), seed=1)
            call()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(repeats):
                call()
            e1.record()
            torch.cuda.synchronize()
            timed[(fuse, lock)] = e0.elapsed_time(e1) / repeats
            b.close()
        (fuse, lock), ms = min(timed.items(), key=lambda kv: kv[1])
        set_row_policy(n, fuse, lock)
        entry = {"fuse": fuse, "lock": lock, "ms": ms, "rows": int(len(idx)),
                 "candidates": {f"fuse={f},lock={lk}": t for (f, lk), t in timed.items()},
                 "tuned_at": time.strftime("%Y-%m-%dT%H:%M:%S")}
        cache[key] = entry
        result[n] = dict(entry, cached=False)
    if use_cache:
        merged = _load_cache()
        merged.update(cache)
        _save_cache(merged)
    return result
