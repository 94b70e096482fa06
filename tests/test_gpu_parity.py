"""GPU parity: the CUDA path (through the C ABI) against the oracle.

* ray generation and the geometry hit are bit-exact (every coordinate);
* the reference's Cone::hit golden cases hold on the device;
* FP64 renders match the oracle at the same tolerances: hit mask and count
  exact, tau within 1e-5, I within 1e-4 (I > 1e-6 max), Q/U/V within
  1e-4 max(I), total flux within 1e-5.
"""
import math

import numpy as np
import pytest

from jetshow_gb300 import _capi as A
from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W
from jetshow_gb300.runtime import mas_to_pc
from helpers import compare_images, flat
from test_oracle import check_cone_cases

pytestmark = pytest.mark.gpu


def planes():
    lg = math.log10(0.1 * 1.8443 * J.pc)
    yield J.ImagePlane((16, 16), lg, lg, 0.1)
    yield J.ImagePlane((24, 40), math.log10(1e-3 * 1.8443 * J.pc), math.log10(1e-1 * 1.8443 * J.pc), 0.1)
    yield J.ImagePlane((10, 7), 17.3, 18.9, 0.05)


def geometries():
    yield J.Cone((0, 0, 0), (0, 0, 1), 0.05, 100 * J.pc)
    yield J.Cone((0, 0, 0), (0, 0, 1), 0.15, 100)          # LOS < half angle: two nappes
    yield J.ParabaloidCone((0, 0, 0), (0, 0, 1), 0.1 * J.pc, 1.0 * J.pc, 100 * J.pc)
    yield J.Parabaloid((0, 0, 0), (0, 0, 1), 0.1 * J.pc, 100 * J.pc)
    yield J.Cylinder((0, 0, 0), (0, 0, 1), 0.5 * J.pc)


def test_plane_rays_bit_exact(ctx, oracle):
    for pl in planes():
        o, d, s = ctx.plane_rays(pl.desc())
        oo, od, os_ = oracle.plane_rays(pl.desc())
        assert np.array_equal(o, oo)
        assert np.array_equal(d, od)
        assert np.array_equal(s, os_)


def test_cone_golden_cases_gpu(ctx):
    check_cone_cases(ctx.hit_rays)


def test_hits_bit_exact(ctx, oracle):
    for pl in planes():
        o, d, _ = oracle.plane_rays(pl.desc())
        dirs = np.tile(d, (o.shape[0], 1))
        for g in geometries():
            jet = J.Jet(g, J.ConstFlatVField(10.0), J.RandomScalarBFieldZ(0.1, 1.0), J.BKNFieldZ(500, 2, True))
            n1, s1, t1 = ctx.trace_plane(jet.desc(), pl.desc())
            n2, s2, t2 = oracle.hit_rays(jet.desc(), o, dirs)
            assert np.array_equal(n1, n2), type(g).__name__
            for k in range(2):
                sel = n2 > k
                assert np.array_equal(s1[sel, k], s2[sel, k]), type(g).__name__
            assert np.array_equal(t1 & ~np.uint32(1), t2 & ~np.uint32(1))


def render_both(ctx, oracle, jet, plane, nu, **kw):
    p = J.make_params(**kw)
    g, st = ctx.render(jet.desc(), plane.desc(), nu, p)
    r = oracle.render(jet.desc(), plane.desc(), nu, p)
    return flat(g), r, st


@pytest.mark.parametrize("output", ["I", "full"])
def test_fp64_conical_c0(ctx, oracle, output):
    jet, plane, nu, kw = W.conical_c0(scale=4)
    kw["output"] = output
    g, r, st = render_both(ctx, oracle, jet, plane, nu, **kw)
    e = compare_images(g, r, full=(output == "full"), tau_max=kw["tau_max"])
    assert e["n_hit"] == st["n_hit_pixels"] > 0


def test_fp64_log_plane_multifreq(ctx, oracle):
    jet, plane, nu, kw = W.conical_c1(scale=16)
    g, r, st = render_both(ctx, oracle, jet, plane, nu, **kw)
    compare_images(g, r, full=True, tau_max=kw["tau_max"])


def test_fp64_parabolic_near_grazing(ctx, oracle):
    jet, plane, nu, kw = W.parabolic_c2(scale=32)
    g, r, st = render_both(ctx, oracle, jet, plane, nu, **kw)
    compare_images(g, r, full=True, tau_max=kw["tau_max"])


def test_fp64_reference_defaults_tangled(ctx, oracle):
    # the model pyjetshow.get_i_image builds (s = 3.42, scalar B, reference tolerances)
    jet = J.Jet(J.Cone((0., 0., 0.), (0., 0., 1.), 0.0165, 100), J.ConstFlatVField(8.0),
                J.RandomScalarBFieldZ(0.1, 1.0), J.BKNFieldZ(500, 2, True), s=3.42)
    lg0, lg1 = math.log10(1e-2 * 1.86 * J.pc), math.log10(1e-1 * 1.86 * J.pc)
    plane = J.ImagePlane((12, 20), lg0, lg1, 0.05)
    g, r, st = render_both(ctx, oracle, jet, plane, [15.4e9 * 1.1], dt_max=J.pc * 0.001 * J.pc)
    compare_images(g, r, full=False, tau_max=1e4)


# Reference cosmology of mas_to_pc (include/utils.h:172) and the pixel
# solid-angle / Jy conversion of get_i_image (src/pyjetshow.cpp:111-169),
# restated here independently of the library.
REF_COSMO = dict(H0=69.32, omega_M=0.2865, omega_V=0.7134130719051658, gamma_nu=8.69280948342326e-05)
MAS_TO_RAD = 4.84813681109536e-09


def ref_pc_in_mas(z):
    """mas_to_rad * D_C(z) / (1 + z) with D_C = (c/H0) 1e6 int_0^z
    ((omega_M + (1+t) gamma_nu)(1+t)^3 + omega_V)^-1/2 dt [pc]
    (src/utils.cpp:195-208, 373-378), by 64-point Gauss-Legendre."""
    x, w = np.polynomial.legendre.leggauss(64)
    t = 0.5 * z * (x + 1.0)
    c = REF_COSMO
    f = ((c["omega_M"] + (1.0 + t) * c["gamma_nu"]) * (1.0 + t) ** 3 + c["omega_V"]) ** -0.5
    d_c = (299792.458 / c["H0"]) * 1e6 * 0.5 * z * np.sum(w * f)
    return MAS_TO_RAD * d_c / (1.0 + z)


def test_pyjetshow_drop_in(ctx, oracle):
    """``import pyjetshow; pyjetshow.get_i_image(...)`` as jetmodel.py:6 and
    :93-96 call it: tau and I in Jy per pixel against the oracle's image of
    the reference's model (Cone(0, +z, half-angle, 100), RandomScalarBFieldZ,
    BKNFieldZ in the plasma frame, ConstFlatVField, s = 3.42, the binding's
    hard-coded tolerances and dt_max = pc * 0.001 scaled by pc once more in
    Observation::run) times the reference's Jy factor
    (1+z)^3 / (1e-23 Omega_pix), at the contract gates in Jy."""
    import pyjetshow

    los, z, n_along, n_across, mas0, mas1 = 0.1, 0.1, 24, 16, 1e-2, 1e-1
    half, B_1, m, K_1, n, Gamma, nu_ghz = 0.05, 0.1, 1.0, 500.0, 2.0, 10.0, 15.4
    tau, img = pyjetshow.get_i_image(los, z, n_along, n_across, mas0, mas1, half, B_1, m, K_1, n, Gamma, nu_ghz)
    assert tau.shape == (n_across, n_along) and img.shape == (n_across, n_along)
    pcm = ref_pc_in_mas(z)
    assert abs(mas_to_pc(z) / pcm - 1.0) < 1e-8  # the library's cosmology is the reference's
    jet = J.Jet(J.Cone((0., 0., 0.), (0., 0., 1.), half, 100), J.ConstFlatVField(Gamma),
                J.RandomScalarBFieldZ(B_1, m), J.BKNFieldZ(K_1, n, True), s=3.42)
    pcl = mas_to_pc(z)
    plane = J.ImagePlane((n_across, n_along), math.log10(mas0 * pcl * J.pc), math.log10(mas1 * pcl * J.pc), los)
    p = J.make_params(n=100, tau_max=1e4, dt_max=J.pc * 0.001 * J.pc, tau_min=1e-10)
    r = oracle.render(jet.desc(), plane.desc(), [nu_ghz * 1e9 * (1 + z)], p)
    _, _, sizes = oracle.plane_rays(plane.desc())
    omega = (sizes / (pcm * J.pc)) ** 2 * MAS_TO_RAD ** 2
    jy = r["I"][0] * omega / (1e-23 * (1 + z) ** 3)
    hit = ((r["status"][0] & A.ST_HIT) != 0)
    assert hit.sum() > 20
    gpu = {"tau": tau.reshape(1, -1), "I": img.reshape(1, -1), "status": r["status"]}
    ref = {"tau": r["tau"], "I": jy.reshape(1, -1), "status": r["status"]}
    e = compare_images(gpu, ref, full=False, tau_max=1e4)
    assert e["n_hit"] == int(hit.sum())
    assert img.max() > 0
