"""The adjoint gradient (tfq_adj_grad) checked against gradients taken from
the forward kernel itself, on rows of the adjoint benchmark's shape: 16
qubits, depth 10 hardware-efficient ansatz (Ry, Rz per qubit per layer, then
a CNOT ladder), 320 symbols with values U[0, 2pi), one transverse-field Ising
observable with 31 terms.

Two independent differentiators, both computed with the repo's own
expectation op on shifted symbol values (one batch row per shift):
- central finite differences, eps = 1e-3: the reference's CentralDifference
  differentiator (python/differentiators/linear_combination.py:251), with the
  step taken as the float64 difference of the float32 values the op sees;
- the parameter-shift rule: the reference's ParameterShift differentiator
  (python/differentiators/parameter_shift.py:22). Every symbol here drives one
  XPow/YPow/ZPow-type gate with exponent t = x * s (s = round(1/pi, 6), the
  serialized scalar). Its two eigenphases differ by pi*t, so
  f(t) = a + b cos(pi t) + c sin(pi t) and
  df/dx = s * (pi/2) * (f(t + 1/2) - f(t - 1/2)), a shift of x by 0.5/s.

Tolerances, relative to max(1, max|grad|) (the gradients here are a few
tenths):
- parameter shift against the exact-derivative adjoint (grad_rule=1): 2e-6.
  Both are exact rules, and only float32 rounding of the state, of
  x +- 0.5/s and of x*s separates them (measured on GB300: 2.8e-7);
- parameter shift against the reference's finite-difference gradient gates
  (grad_rule=0, eps = 5e-3 inside the gate): 5e-5.  The gate rule's
  (G(x+eps) - G(x-eps)) / 2eps in float32 loses about 6e-6 relative to
  cancellation, besides its sin(pi eps s)/(pi eps s) truncation (measured:
  9.3e-6);
- central differences against both adjoint rules: 3e-4.  With eps = 1e-3
  in float32, the 1e-7 relative rounding of the 31-term expectation and of
  x +- eps (spacing 2.4e-7 near 2pi) is divided by 2e-3 (measured: 5.8e-5).
"""

import numpy as np
import pytest

from quantum_gb300 import ops, workloads

pytestmark = pytest.mark.gpu

SCALAR = np.float32(0.318310)  # the serialized exponent scalar of rx/ry/rz


@pytest.fixture(scope="module")
def hea():
    w = workloads.adjoint_hea(batch=2, n=16, depth=10, seed=7)
    prog, ps = w["programs"][0], w["pauli_sums"][0]
    names, vals = w["symbol_names"], w["symbol_values"]
    P = len(names)
    assert P == 320
    g_fd = ops.tfq_adj_grad(w["programs"], names, vals, w["pauli_sums"],
                            np.ones((2, 1), np.float32), grad_rule=0)
    g_ex = ops.tfq_adj_grad(w["programs"], names, vals, w["pauli_sums"],
                            np.ones((2, 1), np.float32), grad_rule=1)
    return dict(prog=prog, ps=ps, names=names, vals=vals, P=P, g_fd=g_fd, g_ex=g_ex)


def _shifted_expectations(h, row, delta):
    """f(x + delta e_j) and f(x - delta e_j) for every symbol j, one batch of
    2P rows through the expectation op; also the float64 steps actually
    taken after float32 rounding."""
    P = h["P"]
    x = h["vals"][row]
    plus = np.repeat(x[None, :], P, axis=0)
    minus = plus.copy()
    idx = np.arange(P)
    plus[idx, idx] = (x + np.float32(delta)).astype(np.float32)
    minus[idx, idx] = (x - np.float32(delta)).astype(np.float32)
    vals = np.concatenate([plus, minus]).astype(np.float32)
    e = ops.tfq_simulate_expectation([h["prog"]] * (2 * P), h["names"], vals,
                                     [h["ps"]] * (2 * P))[:, 0].astype(np.float64)
    step = plus[idx, idx].astype(np.float64) - minus[idx, idx].astype(np.float64)
    return e[:P], e[P:], step, plus[idx, idx], minus[idx, idx]


@pytest.mark.parametrize("row", [0, 1])
def test_adjoint_matches_central_differences(hea, row):
    fp, fm, step, _, _ = _shifted_expectations(hea, row, 1e-3)
    fd = (fp - fm) / step
    scale = max(1.0, float(np.abs(hea["g_ex"][row]).max()))
    assert np.abs(fd).max() > 0.05  # a nonzero gradient is being compared
    print(f"row {row}: central differences vs adjoint: exact rule "
          f"{np.abs(hea['g_ex'][row] - fd).max():.2e}, reference rule "
          f"{np.abs(hea['g_fd'][row] - fd).max():.2e}")
    np.testing.assert_allclose(hea["g_ex"][row], fd, atol=3e-4 * scale, rtol=0)
    np.testing.assert_allclose(hea["g_fd"][row], fd, atol=3e-4 * scale, rtol=0)


@pytest.mark.parametrize("row", [0, 1])
def test_adjoint_matches_parameter_shift(hea, row):
    delta = 0.5 / float(SCALAR)
    fp, fm, _, xp, xm = _shifted_expectations(hea, row, delta)
    # the exponent shifts the op actually applied: float32 x * s on both sides
    x = hea["vals"][row]
    t0 = (x * SCALAR).astype(np.float64)
    tp = (xp * SCALAR).astype(np.float64) - t0
    tm = t0 - (xm * SCALAR).astype(np.float64)
    assert np.abs(tp - 0.5).max() < 1e-6 and np.abs(tm - 0.5).max() < 1e-6
    ps = float(SCALAR) * (np.pi / 2) * (fp - fm)
    scale = max(1.0, float(np.abs(ps).max()))
    assert np.abs(ps).max() > 0.05
    print(f"row {row}: parameter shift vs adjoint: exact rule "
          f"{np.abs(hea['g_ex'][row] - ps).max():.2e}, reference rule "
          f"{np.abs(hea['g_fd'][row] - ps).max():.2e}")
    np.testing.assert_allclose(hea["g_ex"][row], ps, atol=2e-6 * scale, rtol=0)
    np.testing.assert_allclose(hea["g_fd"][row], ps, atol=5e-5 * scale, rtol=0)
