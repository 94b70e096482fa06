"""CPU tests of the oracle: the reference's own Cone::hit golden cases
(tests/simple_test.cpp:17-101), the integrator's known answers and the
transfer equations' analytic solutions for constant coefficients."""
import json
import math
import os

import numpy as np
import pytest
import scipy.linalg

from jetshow_gb300 import _capi as A
from jetshow_gb300 import jet as J

HERE = os.path.dirname(os.path.abspath(__file__))


def cone_model(angle, scale, origin=(0, 0, 0), direction=(0, 0, 1)):
    jet = J.Jet(J.Cone(origin, direction, angle, scale), J.ConstFlatVField(10.0),
                J.RandomScalarBFieldZ(0.1, 1.0), J.BKNFieldZ(500, 2, True))
    return jet.desc()


def load_cases():
    with open(os.path.join(HERE, "golden", "cone_hit_cases.json")) as fh:
        return json.load(fh)


def check_cone_cases(hit_fn):
    G = load_cases()
    c = G["cone"]
    model = cone_model(c["angle"], c["scale"], c["origin"], c["direction"])
    cases = G["cases"]
    o = np.array([k["origin"] for k in cases])
    d = np.array([k["direction"] for k in cases])
    nseg, seg, st = hit_fn(model, o, d)
    tol = G["tolerance_sq"]
    for i, k in enumerate(cases):
        assert nseg[i] == k["n"], (i, k["kind"], nseg[i])
        if k["n"]:
            pin, pout = seg[i, 0, 0], seg[i, 0, 1]
            assert np.sum((pin - np.array(k["point_in"])) ** 2) <= tol, (i, k["kind"], pin)
            assert np.sum((pout - np.array(k["point_out"])) ** 2) <= tol, (i, k["kind"], pout)


def test_cone_golden_cases(oracle):
    check_cone_cases(oracle.hit_rays)


def test_dense_output_order(oracle):
    # the continuous extension is 4th order: local error O(h^5)
    e1 = abs(oracle.lib().jo_test_dense_error(0.2, 0.5))
    e2 = abs(oracle.lib().jo_test_dense_error(0.1, 0.5))
    assert e1 > 0 and 20 < e1 / e2 < 45, (e1, e2)
    # at theta = 1 it is the 5th-order step itself: local error O(h^6)
    f1 = abs(oracle.lib().jo_test_dense_error(0.2, 1.0))
    f2 = abs(oracle.lib().jo_test_dense_error(0.1, 1.0))
    assert 50 < f1 / f2 < 80, (f1, f2)


@pytest.mark.parametrize("a,b,L", [(-1.0, 1.0, 3.0), (-50.0, 2.0, 1.0), (0.3, 0.1, 2.0)])
def test_linear_known_answer(oracle, a, b, L):
    import ctypes as C
    ns = C.c_int64()
    x = oracle.lib().jo_test_linear_controlled(a, b, L, L / 100, 1e-12, 1e-12, C.byref(ns))
    exact = b / a * (math.exp(a * L) - 1.0)
    assert abs(x - exact) <= 1e-9 * max(1.0, abs(exact))
    assert ns.value > 0


def test_mas_to_pc_values(oracle):
    # flat LCDM (H0 70, Om 0.3) and the reference's WMAP9-like default at z = 0.1
    flat = A.Cosmology(H0=70.0, omega_M=0.3, omega_V=0.7, gamma_nu=0.0)
    assert abs(oracle.mas_to_pc(0.1, flat) - 1.8443) < 2e-4
    assert abs(oracle.mas_to_pc(0.1) - 1.8643) < 2e-4


def const_model(b0=0.5, n0=1e3, gamma=1.0, s=2.5, thermal=0.0, angle=0.3, gamma_min=10.0):
    """Constant coefficients: B = (0, 0, b0), n = n0, v = 0 (D = 1)."""
    jet = J.Jet(J.Cone((0, 0, 0), (0, 0, 1), angle, J.pc), J.ConstFlatVField(gamma),
                J.ConstCylinderBField(b0, 0.0, True), J.ConstNField(n0, True), s=s, gamma_min=gamma_min,
                thermal_fraction=thermal)
    return jet.desc()


def small_plane(n=8, los=0.5, mas=2.0):
    lg = math.log10(mas * 1.8443 * J.pc)
    return J.ImagePlane((n, n), lg, lg, los).desc()


def test_constant_coefficients_I(oracle):
    m = const_model()
    plane = small_plane()
    nu = np.array([5e9])
    p = J.make_params(tau_atol=1e-12, tau_rtol=1e-12, atol=1e-30, rtol=1e-12, output="I", tau_max=1e30)
    r = oracle.render(m, plane, nu, p)
    hit = (r["status"][0] & 1) != 0
    assert hit.sum() > 4
    # coefficients along the LOS of the plane (constant in space)
    o, d, _ = oracle.plane_rays(plane)
    k = oracle.coefficients(m, [0, 0, 1e18], -d, nu[0])
    kI, eI = k[0], k[7]
    L = r["l"][0][hit]
    tau_exact = kI * L
    I_exact = eI / kI * (1.0 - np.exp(-kI * L))
    assert np.max(np.abs(r["tau"][0][hit] - tau_exact) / tau_exact) < 1e-9
    assert np.max(np.abs(r["I"][0][hit] - I_exact) / I_exact) < 1e-9


def test_constant_coefficients_full_stokes(oracle):
    # Faraday depth ~20 rad, tau ~2, conversion depth ~3 along the longest ray
    m = const_model(b0=0.2, n0=10.0, thermal=1e-4, gamma_min=30.0)
    plane = small_plane(mas=1.0)
    nu = np.array([5e9])
    p = J.make_params(tau_atol=1e-12, tau_rtol=1e-12, atol=1e-40, rtol=1e-12, output="full", tau_max=1e30)
    r = oracle.render(m, plane, nu, p)
    hit = np.nonzero((r["status"][0] & 1) != 0)[0]
    o, d, _ = oracle.plane_rays(plane)
    kI, kQ, kU, kV, kF, kC, hQ, eI, eQ, eU, eV = oracle.coefficients(m, [0, 0, 1e18], -d, nu[0])
    assert kF != 0 and kC != 0 and kV != 0
    K = np.array([[kI, kQ, kU, kV], [kQ, kI, kF, hQ], [kU, -kF, kI, kC], [kV, -hQ, -kC, kI]])
    eta = np.array([eI, eQ, eU, eV])
    worst = 0.0
    for pix in hit:
        L = r["l"][0][pix]
        x = np.linalg.solve(K, (np.eye(4) - scipy.linalg.expm(-K * L)) @ eta)
        got = np.array([r[k][0][pix] for k in "IQUV"])
        worst = max(worst, np.max(np.abs(got - x)) / abs(x[0]))
    assert worst < 1e-8, worst


def test_plane_layout(oracle):
    plane = J.ImagePlane((6, 5), 17.0, 18.0, 0.3).desc()
    o, d, s = oracle.plane_rays(plane)
    s = s.reshape(6, 5)
    assert np.allclose(s[0], np.logspace(17, 18, 5), rtol=1e-14)
    o = o.reshape(6, 5, 3)
    # rows: 3 positive offsets flipped, then 3 negated ones
    assert np.all(o[:3, :, 1] > 0) and np.all(o[3:, :, 1] < 0)
    assert np.array_equal(o[2, :, 1], -o[3, :, 1])
    assert np.allclose(o[2, :, 1], 0.5 * s[0])
    assert np.allclose(d, [-math.sin(0.3), 0, -math.cos(0.3)])


def test_scalar_field_polarisation_is_zero(oracle):
    jet = J.Jet(J.Cone((0, 0, 0), (0, 0, 1), 0.05, 100 * J.pc), J.ConstFlatVField(10.0),
                J.RandomScalarBFieldZ(0.1, 1.0), J.BKNFieldZ(500, 2, True), s=2.5)
    lg = math.log10(0.4 * 1.8443 * J.pc)
    plane = J.ImagePlane((8, 8), lg, lg, 0.1).desc()
    r = oracle.render(jet.desc(), plane, [15e9], J.make_params(output="full"))
    ri = oracle.render(jet.desc(), plane, [15e9], J.make_params(output="I"))
    assert np.all(r["Q"] == 0) and np.all(r["U"] == 0) and np.all(r["V"] == 0)
    assert np.array_equal(r["I"], ri["I"])


def _rays_through(n, seed, extent_pc, los):
    """Image-plane-like rays (direction (-sin los, 0, -cos los)) with
    origins spread over the jet's neighbourhood."""
    rng = np.random.default_rng(seed)
    o = np.column_stack([np.zeros(n), rng.uniform(-0.2, 0.2, n) * extent_pc,
                         rng.uniform(0.0, 1.0, n) * extent_pc]) * J.pc
    d = np.tile([-math.sin(los), 0.0, -math.cos(los)], (n, 1))
    return o, d


def test_hit_points_lie_on_the_surfaces(oracle):
    """Known answer of the geometry: finite chord end points satisfy their
    surface's quadric to 1e-12 relative -- the cone (d.(p-o))^2 = cos^2(a)
    |p-o|^2 (src/Cone.cpp:56-118), the cylinder |w|^2 = r/pc in pc units
    (the reference's c0, src/Cylinder.cpp:53) and the paraboloid x^2 + y^2 =
    (r0^2/pc) z (src/Geometry.cpp:28-69)."""
    field = (J.ConstFlatVField(10.0), J.RandomScalarBFieldZ(0.1, 1.0), J.BKNFieldZ(500, 2, True))
    alpha = 0.05
    cases = {
        "cone": (J.Cone((0, 0, 0), (0, 0, 1), alpha, 100 * J.pc),
                 lambda p: ((p[:, 2] ** 2 - math.cos(alpha) ** 2 * np.sum(p ** 2, axis=1))
                            / np.sum(p ** 2, axis=1))),
        "cylinder": (J.Cylinder((0, 0, 0), (0, 0, 1), 0.5 * J.pc),
                     lambda p: ((p[:, 0] ** 2 + p[:, 1] ** 2) / J.pc ** 2 - 0.5 * J.pc / J.pc) / (0.5 * J.pc / J.pc)),
        "paraboloid": (J.Parabaloid((0, 0, 0), (0, 0, 1), 0.1 * J.pc, 100 * J.pc),
                       lambda p: ((p[:, 0] ** 2 + p[:, 1] ** 2 - (0.1 * J.pc) ** 2 / J.pc * p[:, 2])
                                  / (p[:, 0] ** 2 + p[:, 1] ** 2))),
    }
    for name, (geo, residual) in cases.items():
        o, d = _rays_through(4000, 1, 20.0, 0.1)
        nseg, seg, st = oracle.hit_rays(J.Jet(geo, *field).desc(), o, d)
        fin = nseg == 1
        # chords shorter than the 100 pc (half-)infinite paths are finite on both ends
        fin &= np.linalg.norm(seg[:, 0, 1] - seg[:, 0, 0], axis=1) < 50 * J.pc
        assert fin.sum() > 200, name
        for end in (0, 1):
            r = residual(seg[fin, 0, end])
            assert np.max(np.abs(r)) < 1e-12, (name, end, np.max(np.abs(r)))


def test_optically_thin_limit(oracle):
    """Known answer of the transfer: with a density so low that tau ~ 1e-9,
    I equals the path integral of eta_I to that order."""
    jet = J.Jet(J.Cone((0, 0, 0), (0, 0, 1), 0.05, 100 * J.pc), J.ConstFlatVField(10.0),
                J.HelicalConicalBField(0.1, 1.0, math.pi / 4, True), J.BKNField(5e-6, 2.0, True), s=2.5,
                gamma_min=10.0)
    m = jet.desc()
    lg = math.log10(0.4 * 1.8443 * J.pc)
    plane = J.ImagePlane((8, 8), lg, lg, 0.1).desc()
    nu = np.array([15.4e9 * 1.1])
    p = J.make_params(tau_atol=1e-30, tau_rtol=1e-12, atol=1e-40, rtol=1e-11, output="I", tau_max=1e30,
                      tau_min=1e-300)
    r = oracle.render(m, plane, nu, p)
    o, d, _ = oracle.plane_rays(plane)
    nseg, seg, _ = oracle.hit_rays(m, o, np.tile(d, (o.shape[0], 1)))
    hit = np.nonzero(nseg == 1)[0]
    assert hit.size > 4
    assert np.max(r["tau"][0][hit]) < 1e-6
    for pix in hit[:3]:
        a, b = seg[pix, 0, 0], seg[pix, 0, 1]
        s = np.linspace(0.0, 1.0, 100001)
        eta = np.array([oracle.coefficients(m, a + t * (b - a), -d, nu[0])[7] for t in s])
        integral = np.trapezoid(eta, s) * np.linalg.norm(b - a)
        assert abs(r["I"][0][pix] - integral) / integral < 1e-6, (pix, r["I"][0][pix], integral)


def test_visibility_direct_sum_known_answers():
    """The FP64 direct sum of the visibility tests: a single pixel gives
    F exp(-2 pi i (u' x + v' y)) times the shift; a symmetric pair about the
    phase centre gives a real visibility 2 F cos(2 pi u' x); the pixel
    centres follow the image's running-sum / half-integer layout."""
    import sys
    import os
    sys.path.insert(0, os.path.dirname(__file__))
    from vis_oracle import direct_sum, pixel_centres
    across, along = pixel_centres([1.0, 2.0, 4.0], 4)
    assert np.allclose(along[0], [0.5, 2.0, 5.0])
    assert np.allclose(across[:, 0], [1.5, 0.5, -0.5, -1.5]) and np.allclose(across[:, 2], [6, 2, -2, -6])
    uv = np.array([[0.0, 0.0], [0.25, 0.0], [0.1, 0.3]])
    v = direct_sum([2.0], [-3.0], [5.0], uv, 1.0, dx=0.5, dy=0.0, rot=0.0)
    ph = uv[:, 0] * 3.0 + uv[:, 1] * 5.0 + uv[:, 0] * 0.5
    assert np.allclose(v, 2.0 * np.exp(-2j * np.pi * ph), atol=1e-14)
    v2 = direct_sum([1.0, 1.0], [-2.0, 2.0], [0.0, 0.0], uv, 1.0)
    assert np.allclose(v2.imag, 0, atol=1e-14) and np.allclose(v2.real, 2 * np.cos(2 * np.pi * uv[:, 0] * 2.0))
    # a rotation by pi/2 maps u' = v, v' = -u
    v3 = direct_sum([1.0], [-1.0], [0.0], np.array([[0.0, 0.2]]), 1.0, rot=np.pi / 2)
    assert np.allclose(v3, np.exp(-2j * np.pi * 0.2), atol=1e-14)
