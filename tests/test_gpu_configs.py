"""Parity at the benchmark configurations' own sizes (GPU, through the C ABI),
against the complex128 oracle:

- expectation, 32 circuits x 12 qubits, 20 layers of Rx Ry Rz + CZ
  brick-wall, 4 observables: every row within 1e-5 absolute;
- uneven batch, 4096 random circuits of 4-20 qubits and 5-40 layers, sum Z
  plus 1000 samples per circuit, all in one call each: sum Z within 1e-5 on
  rows of every qubit count, and the samples of one row per qubit-count
  bucket against the oracle's |psi|^2 (chi-squared, p > 1e-3);
- a 24-qubit grid circuit (4 x 6 grid, depth 24, sqrt(X)/sqrt(Y)/sqrt(W) +
  fSim), forward passes as 5-qubit tensor-core blocks in split 3xTF32: the
  state and sum Z against the oracle;
- noisy trajectories, Ry Rz + CZ brick-wall with depolarizing(0.01) after
  every gate, 2000 trajectories per circuit: the trajectory mean within 5
  standard errors of the exact density-matrix value, the standard error
  taken from 16 independent repeats.

The 1e-5 bound is the absolute error the reference's own op tests allow
(circuit_execution_ops_test.py uses atol=1e-5 against cirq).  Large oracle
runs go through oracle/fast128.py (the oracle's complex128 arithmetic in C)."""

import numpy as np
import pytest

from oracle import fast128 as F
from oracle import tfq_oracle as O
from quantum_gb300 import _native, ops, workloads
from tests.stats import bits_to_index, chi2_pvalue

pytestmark = pytest.mark.gpu


def test_c1_every_row_within_1e5():
    w = workloads.expectation_layers(32, 12, 20, seed=1)
    got = ops.tfq_simulate_expectation(w["programs"], w["symbol_names"],
                                       w["symbol_values"], w["pauli_sums"])
    want = O.simulate_expectation(w["programs"], w["symbol_names"],
                                  w["symbol_values"], w["pauli_sums"])
    assert got.shape == (32, 4)
    err = np.abs(got - want).max()
    print(f"c1 max abs error {err:.3e}")
    assert err <= 1e-5


@pytest.fixture(scope="module")
def c3():
    w = workloads.uneven_batch(4096, 4, 20, 5, 40, seed=1)
    b = ops.Batch(w["programs"], [], w["pauli_sums"], ops.KIND_FORWARD)
    vals = np.zeros((4096, 0), np.float32)
    e = b.expectation(vals)
    s = b.samples(vals, 1000, seed=11)
    b.close()
    return w, e, s


def _c3_rows(w, per_n_small=3, per_n_large=1):
    """Rows to check: the shallowest few of every qubit count (oracle cost
    grows with 2^n x depth)."""
    ns = np.array(w["n_per_row"])
    rows = []
    for n in range(4, 21):
        idx = np.nonzero(ns == n)[0]
        depth = [len(w["programs"][i]) for i in idx]  # bytes grow with depth
        take = per_n_small if n <= 16 else per_n_large
        rows += [int(idx[k]) for k in np.argsort(depth)[:take]]
    return rows


def test_c3_expectation_rows_of_every_qubit_count(c3):
    w, e, _ = c3
    errs = []
    for r in _c3_rows(w):
        want = F.simulate_expectation_row(w["programs"][r], [], np.zeros(0, np.float32),
                                          w["pauli_sums"][r])
        errs.append(abs(float(e[r, 0]) - want[0]))
    print(f"c3 sum-Z max abs error over {len(errs)} rows: {max(errs):.3e}")
    assert max(errs) <= 1e-5


def test_c3_samples_chi2_per_bucket(c3):
    w, _, s = c3
    ns = np.array(w["n_per_row"])
    maxn = s.shape[2]
    assert maxn == 20 and s.shape[:2] == (4096, 1000)
    for lo, hi in ((4, 8), (9, 12), (13, 16), (17, 20)):
        idx = np.nonzero((ns >= lo) & (ns <= hi))[0]
        r = int(min(idx, key=lambda i: len(w["programs"][i])))
        n = int(ns[r])
        # leading max_n - n columns are padding
        assert (s[r, :, :maxn - n] == -2).all()
        assert set(np.unique(s[r, :, maxn - n:])) <= {0, 1}
        _, _, psi = F.simulate_state_row(w["programs"][r], [], np.zeros(0, np.float32))
        probs = np.abs(psi) ** 2
        counts = np.bincount(bits_to_index(s[r], n), minlength=2 ** n)
        p, chi2, bins = chi2_pvalue(counts, probs, 1000)
        print(f"c3 bucket {lo}-{hi}: row {r} n={n} chi2={chi2:.1f} bins={bins} p={p:.3g}")
        assert p > 1e-3


def test_c4_24_qubit_tensor_core_state_vs_oracle():
    w = workloads.grid_fsim(4, 6, 24, seed=1)
    prev = _native.set_tensor_core_gates(2)
    try:
        b = ops.Batch(w["programs"], [], w["pauli_sums"], ops.KIND_FORWARD)
        vals = np.zeros((1, 0), np.float32)
        st = b.state(vals)[0].astype(np.complex128)
        blocks = _native.tc_blocks(b._h, 0)
        e = float(b.expectation(vals)[0, 0])
        status = _native.tc_status(b._h)
        b.close()
    finally:
        _native.set_tensor_core_gates(prev)
    assert blocks > 0, "the 24-qubit row must run as tensor-core blocks"
    assert status == 0
    n, index, psi = F.simulate_state_row(w["programs"][0], [], np.zeros(0, np.float32))
    assert n == 24
    want_e = F.expectation(psi, n, O.decode_paulisum(w["pauli_sums"][0][0]), index)
    d = st - psi
    max_amp = float(np.abs(d).max())
    l2 = float(np.linalg.norm(d))
    print(f"c4 24q: {blocks} blocks, max|d amp| {max_amp:.3e}, ||d||_2 {l2:.3e}, "
          f"sum Z {e:.7f} vs {want_e:.7f}")
    # amplitudes are ~2^-12 = 2.4e-4; float32 rounding over ~60 block
    # sweeps stays far below 1e-6 per amplitude and 1e-4 in 2-norm
    assert max_amp <= 1e-6
    assert l2 <= 1e-4
    assert abs(e - want_e) <= 1e-5


@pytest.mark.parametrize("n,rows", [(10, 2), (14, 1)])
def test_c5_trajectory_mean_vs_exact_density_matrix(n, rows):
    w = workloads.noisy_brickwall(rows, n, 15, 0.01, seed=3)
    b = ops.Batch(w["programs"], [], w["pauli_sums"], ops.KIND_NOISY)
    vals = np.zeros((rows, 0), np.float32)
    reps = np.full((rows, 1), 2000, np.int32)
    means = np.stack([b.noisy_expectation(vals, reps, seed=100 + k)[:, 0]
                      for k in range(16)])
    b.close()
    exact = F.noisy_expectation_exact(w["programs"], [], vals, w["pauli_sums"])[:, 0]
    se = means.std(axis=0, ddof=1)  # standard error of one 2000-trajectory mean
    for r in range(rows):
        dev = abs(float(means[0, r]) - exact[r])
        print(f"c5 n={n} row {r}: 2000-trajectory mean {means[0, r]:.5f}, exact "
              f"{exact[r]:.5f}, standard error {se[r]:.4f}, |d|/se {dev / se[r]:.2f}")
        assert dev <= 5 * se[r] + 1e-4
        # all 16 x 2000 trajectories together
        dev_all = abs(float(means[:, r].mean()) - exact[r])
        assert dev_all <= 5 * se[r] / 4 + 1e-4
