"""Stripe mode in the oracle (CPU): Observation::run_stripe
(src/Observation.cpp:310-347) with integrate_tau's constant-step RK4
(src/Observation.cpp:55-123) -- exact for constant coefficients, the stop
at the first step past tau_max, the stripe's pixels (Image::getStripe,
src/Image.cpp:31-41), and agreement with the adaptive tau pass."""
import math

import numpy as np

from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W
from test_oracle import const_model, small_plane


def stripe_pixels(plane):
    na, nl = int(plane.n_across), int(plane.n_along)
    return (na // 2) * nl + np.arange(nl // 2, nl)


def test_constant_coefficients_exact(oracle):
    m = const_model()
    plane = small_plane(n=16)
    nu = 5e9
    k = oracle.coefficients(m, [0, 0, 1e18], -oracle.plane_rays(plane)[1], nu)[0]
    ref = oracle.render(m, plane, [nu], J.make_params(tau_max=1e30), pix=stripe_pixels(plane))
    L = ref["l"][0]
    hit = L > 0
    assert hit.sum() >= 3
    s = oracle.stripe(m, plane, nu, n=50, tau_max=1e30)
    # RK4 integrates a constant rate exactly: tau = k L
    np.testing.assert_allclose(s[hit], k * L[hit], rtol=1e-12)
    assert np.all(s[~hit] == 0.0)
    # stopped at the first step whose tau reaches tau_max: tau = ceil(tau_max / (k dt)) k dt
    tau_max = 0.37 * float(np.max(k * L[hit]))
    s = oracle.stripe(m, plane, nu, n=50, tau_max=tau_max)
    for i in np.nonzero(hit)[0]:
        step = k * L[i] / 50
        expect = k * L[i] if k * L[i] < tau_max else math.ceil(tau_max / step - 1e-9) * step
        assert abs(s[i] - expect) <= 1e-9 * expect, (i, s[i], expect)


def test_stripe_matches_adaptive_tau(oracle):
    jet, plane, nu, _ = W.conical_c0(scale=4)
    m, pd = jet.desc(), plane.desc()
    s = oracle.stripe(m, pd, nu[0], n=4000, tau_max=1e30)
    ref = oracle.render(m, pd, nu, J.make_params(tau_max=1e30, tau_atol=1e-30, tau_rtol=1e-11),
                        pix=stripe_pixels(pd))
    hit = ref["tau"][0] > 0
    assert hit.sum() >= 4
    np.testing.assert_allclose(s[hit], ref["tau"][0][hit], rtol=1e-6)
    assert np.all(s[~hit] == 0.0)
