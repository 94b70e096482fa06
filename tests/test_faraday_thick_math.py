"""The approximations of the Faraday-thick mode of the mixed IQUV pass,
checked on the CPU against the exact solution of the transfer equation with
frozen coefficients (a matrix exponential of the reference's full-Stokes
system, src/System.cpp:41-63, in the lab frame with k_U = eta_U = 0):

* the lab-frame polarisation Pi = Q + iU relaxes at lambda = k_I - i k_F
  towards S / lambda, S = (eta_Q - k_Q I) - i k_C V;
* in the frame rotating with chi' = k_F the transient d = (q + iu) -
  e^{-i chi} S / lambda only decays, d(t) = d(0) e^{-k_I t}, when S is
  constant (the mode carries it that way);
* leaving the transient's rotating share out of I and V moves them by at
  most ~max(|k_Q|, |k_C|) |d(0)| / |lambda| (the bound the mode's entry and
  every step check).
"""
import numpy as np
import pytest

scipy_linalg = pytest.importorskip("scipy.linalg")


def transfer_matrix(kI, kQ, kV, kF, kC):
    # dx/dt = eps - K x, x = (I, Q, U, V)
    return np.array([[kI, kQ, 0.0, kV],
                     [kQ, kI, kF, 0.0],
                     [0.0, -kF, kI, kC],
                     [kV, 0.0, -kC, kI]])


def exact(K, eps, x0, t):
    """x(t) of dx/dt = eps - K x: x_eq + e^{-K t} (x0 - x_eq)."""
    xeq = np.linalg.solve(K, eps)
    return xeq + scipy_linalg.expm(-K * t) @ (x0 - xeq)


CASES = [
    # kI, kQ, kV, kF, kC, eta_I, eta_Q, eta_V: Faraday rotation 100x .. 3000x absorption
    (1.0, 0.7, 0.01, 100.0, 0.05, 1.0, 0.7, 0.01),
    (0.3, 0.2, -0.005, -900.0, 0.3, 0.5, 0.35, -0.004),
    (2.0, 1.3, 0.02, 6000.0, 1.0, 3.0, 2.0, 0.02),
]


@pytest.mark.parametrize("case", CASES)
def test_polarisation_relaxes_to_the_quasi_static_value(case):
    kI, kQ, kV, kF, kC, eI, eQ, eV = case
    K = transfer_matrix(kI, kQ, kV, kF, kC)
    eps = np.array([eI, eQ, 0.0, eV])
    x = exact(K, eps, np.zeros(4), 40.0 / kI)  # 40 absorption lengths: at equilibrium
    lam = kI - 1j * kF
    S = (eQ - kQ * x[0]) - 1j * kC * x[3]
    pi = x[1] + 1j * x[2]
    assert abs(pi - S / lam) <= 1e-12 * abs(x[0])


@pytest.mark.parametrize("case", CASES)
def test_rotating_frame_transient_only_decays(case):
    """With I and V held (k_Q = k_C = 0 couplings of Pi into them, and S
    frozen), d(t) = d(0) e^{-k_I t} exactly in the rotating frame."""
    kI, kQ, kV, kF, kC, eI, eQ, eV = case
    I0, V0 = 0.8 * eI / kI, 0.1 * eV / kI
    lam = kI - 1j * kF
    S = (eQ - kQ * I0) - 1j * kC * V0
    pi0 = 0.3 * abs(S) / kI * np.exp(0.7j)  # a transient far from S / lambda
    d0 = pi0 - S / lam
    for t in (0.01 / kI, 0.5 / kI, 3.0 / kI):
        # Pi' = -lambda Pi + S with S frozen
        pi = S / lam + (pi0 - S / lam) * np.exp(-lam * t)
        chi = kF * t
        d = np.exp(-1j * chi) * (pi - S / lam)
        assert abs(d - d0 * np.exp(-kI * t)) <= 1e-12 * abs(d0)


@pytest.mark.parametrize("case", CASES)
def test_left_out_coupling_of_the_transient_is_bounded(case):
    """Start (Q, U) away from its quasi-static value and integrate I and V
    once with the full coupling and once with Pi = S / lambda + the decaying
    transient but without the transient's share in I and V: the two differ
    by at most ~2 max(|k_Q|, |k_C|) |d(0)| / |lambda| at every time."""
    kI, kQ, kV, kF, kC, eI, eQ, eV = case
    K = transfer_matrix(kI, kQ, kV, kF, kC)
    eps = np.array([eI, eQ, 0.0, eV])
    lam = kI - 1j * kF
    xeq = np.linalg.solve(K, eps)
    d0 = 1e-3 * abs(xeq[0]) * np.exp(1.1j)
    x0 = xeq.copy()
    x0[1] += d0.real
    x0[2] += d0.imag
    # the mode's model: I, V with Pi = S(I, V) / lambda only (a 2x2 linear
    # system, exact by its own matrix exponential), transient not fed back
    # Re(S / lambda) = (sre kI - sim kF) / |lambda|^2, Im = (sre kF + sim kI) / |lambda|^2,
    # sre = eQ - kQ I, sim = -kC V; I' = eI - kI I - kQ Re - kV V,
    # V' = eV - kI V - kV I + kC Im; written y' = b - a y
    l2 = abs(lam) ** 2
    a = np.array([[kI - kQ * kQ * kI / l2, kV + kQ * kC * kF / l2],
                  [kV + kC * kQ * kF / l2, kI + kC * kC * kI / l2]])
    b = np.array([eI - kQ * eQ * kI / l2, eV + kC * eQ * kF / l2])
    yeq = np.linalg.solve(a, b)
    assert np.allclose(yeq, xeq[[0, 3]], rtol=1e-12, atol=1e-12 * abs(xeq[0]))  # the full system's equilibrium
    bound = 2.0 * max(abs(kQ), abs(kC)) * abs(d0) / abs(lam)
    worst = 0.0
    for t in np.linspace(0.0, 6.0 / kI, 49):
        full = exact(K, eps, x0, t)
        mode = yeq + scipy_linalg.expm(-a * t) @ (x0[[0, 3]] - yeq)
        worst = max(worst, abs(full[0] - mode[0]), abs(full[3] - mode[1]))
    assert worst <= bound * 1.05
    assert worst >= 0.03 * bound  # the bound is of the right size, not vacuous (0.07 .. 0.8 of it here)
