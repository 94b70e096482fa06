"""Stripe mode on the GPU (Observation::run_stripe, src/Observation.cpp:310-347):
the device's FP64 constant-step RK4 tau along half of the central row
against the oracle's, with and without the stop at tau_max, on the conical,
log-plane and ParabaloidCone jets, through the C ABI and the Observation
mirror."""
import numpy as np
import pytest

from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_stripe_device_matches_oracle(ctx, oracle):
    for wl, scale in ((W.conical_c0, 1), (W.conical_c1, 4), (W.parabolic_c2, 16)):
        jet, plane, nu, _ = wl(scale=scale)
        for tau_max in (1e4, 1.0):
            g = ctx.stripe(jet.desc(), plane.desc(), nu[0], n=100, tau_max=tau_max)
            r = oracle.stripe(jet.desc(), plane.desc(), nu[0], n=100, tau_max=tau_max)
            assert g.shape == r.shape
            assert np.array_equal(g == 0, r == 0)
            assert (g > 0).sum() >= 2
            # the k_I evaluations differ only in the last bits of pow on the device
            np.testing.assert_allclose(g, r, rtol=1e-10, atol=0)


def test_observation_stripe_mirror(ctx):
    jet, plane, nu, _ = W.conical_c0()
    obs = J.Observation(jet, plane, nu).run_stripe(100, 1e4, 1e-10, ctx=ctx)
    s = obs.getStripe("tau")
    assert s.shape == (plane.image_size[1] - plane.image_size[1] // 2,)
    assert np.array_equal(s, ctx.stripe(jet.desc(), plane.desc(), nu[0], n=100, tau_max=1e4))
