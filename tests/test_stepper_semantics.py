"""The oracle's adaptive stepper against an independent restatement of the
published method it follows: the Dormand-Prince 5(4) pair (Dormand & Prince,
J. Comp. Appl. Math. 6, 1980) with the first-same-as-last derivative, and
Boost.Odeint's controlled_runge_kutta semantics, which the reference's
steppers use (make_dense_output for the tau pass, src/Observation.cpp:154-156;
make_controlled in integrate_adaptive for the I pass, :262-269):
error = max_i |err_i| / (atol + rtol (|x_i| + |dt| |x'_i|)); a step with
error > 1 is retried with dt max(0.9 error^(-1/3), 0.2); an accepted step
with error < 0.5 grows dt by 0.9 max(error, 5^-5)^(-1/5); the last step is
cut to end on the interval's end.  On dx/dt = a x + b the two must take the
same number of accepted steps and agree on the end value."""
import math

import pytest

C = [0.0, 1 / 5, 3 / 10, 4 / 5, 8 / 9, 1.0, 1.0]
A = [[],
     [1 / 5],
     [3 / 40, 9 / 40],
     [44 / 45, -56 / 15, 32 / 9],
     [19372 / 6561, -25360 / 2187, 64448 / 6561, -212 / 729],
     [9017 / 3168, -355 / 33, 46732 / 5247, 49 / 176, -5103 / 18656],
     [35 / 384, 0.0, 500 / 1113, 125 / 192, -2187 / 6784, 11 / 84]]
B5 = A[6] + [0.0]
B4 = [5179 / 57600, 0.0, 7571 / 16695, 393 / 640, -92097 / 339200, 187 / 2100, 1 / 40]


def integrate(a, b, L, dt0, atol, rtol):
    f = lambda x: a * x + b  # noqa: E731
    t, x, dt = 0.0, 0.0, dt0
    k1 = f(x)
    accepted = 0
    eps = 2.220446049250313e-16
    while L - t > eps:
        if (t + dt) - L > eps:
            dt = L - t
        for _ in range(500):
            k = [k1]
            for s in range(1, 7):
                k.append(f(x + dt * sum(A[s][j] * k[j] for j in range(s))))
            xn = x + dt * sum(B5[j] * k[j] for j in range(7))
            kn = f(xn)
            k[6] = kn
            err = abs(dt * sum((B5[j] - B4[j]) * k[j] for j in range(7)))
            e = err / (atol + rtol * (abs(x) + abs(dt) * abs(k1)))
            if e > 1.0:
                dt *= max(0.9 * e ** (-1 / 3), 0.2)
                continue
            t, x, k1 = t + dt, xn, kn
            if e < 0.5:
                dt *= 0.9 * max(e, 5.0 ** -5) ** (-1 / 5)
            accepted += 1
            break
    return x, accepted


CASES = [(-1.0, 1.0, 3.0, 0.03, 1e-12, 1e-12), (-50.0, 2.0, 1.0, 0.01, 1e-10, 1e-8),
         (0.3, 0.1, 2.0, 0.02, 1e-9, 1e-6), (-5.0, 1.0, 10.0, 0.1, 1e-14, 1e-10),
         (-0.2, 3.0, 40.0, 1.0, 1e-8, 1e-6), (2.0, -1.0, 4.0, 1e-3, 1e-12, 1e-9)]


@pytest.mark.parametrize("case", CASES)
def test_controlled_stepper_takes_the_published_steps(oracle, case):
    import ctypes as Ct
    a, b, L, dt0, atol, rtol = case
    ns = Ct.c_int64()
    got = oracle.lib().jo_test_linear_controlled(a, b, L, dt0, atol, rtol, Ct.byref(ns))
    x, accepted = integrate(a, b, L, dt0, atol, rtol)
    assert ns.value == accepted
    assert abs(got - x) <= 1e-13 * max(1.0, abs(x))
    exact = b / a * (math.exp(a * L) - 1.0)
    assert abs(x - exact) <= 1e3 * rtol * max(1.0, abs(exact))
