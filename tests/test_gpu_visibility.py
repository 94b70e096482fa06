"""The visibility step on the device (jsh_observation_visibilities) against
an FP64 direct sum over the same rendered image (tests/vis_oracle.py).

The reference's gate is FINUFFT's requested precision, eps 1e-6
(fourier.py:40-94): the device sum must be within 1e-6 of the exact sum in
relative l2 norm over the (u, v) points, and within 1e-6 of max |V| at every
point.  Phases reach hundreds of cycles (long baselines, the full image
extent), so the test exercises the phase reduction.
"""
import math

import numpy as np
import pytest

from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W
from vis_oracle import direct_sum, pixel_centres

pytestmark = pytest.mark.gpu

MAS_TO_RAD = 4.84813681109536e-09


def uv_points(n, umax, seed=3):
    rng = np.random.default_rng(seed)
    r = umax * np.sqrt(rng.random(n))
    t = rng.uniform(0, 2 * np.pi, n)
    uv = np.column_stack([r * np.cos(t), r * np.sin(t)])
    uv[:8] = [[0, 0], [1e6, 0], [0, 1e6], [-3e7, 2e7], [umax, 0], [0, umax], [-umax, 0], [0, -umax]]
    return uv


@pytest.mark.parametrize("case", ["c1_log", "c0_uniform"])
def test_visibilities_match_direct_sum(ctx, case):
    if case == "c1_log":
        jet, plane, nu, _ = W.conical_c1(scale=8, n_freq=2)   # 64 x 128, lg mas -3 .. -1
    else:
        jet, plane, nu, _ = W.conical_c0(scale=2)             # 64 x 64 uniform
    p = J.make_params(precision="mixed", schedule="persistent", **W.ACCURATE_KW)
    img, _ = ctx.render(jet.desc(), plane.desc(), nu, p)
    pcm = W.pc_per_mas()
    rad_per_cm = MAS_TO_RAD / (pcm * J.pc)
    jy = 1e23 / (1 + W.Z) ** 3 * rad_per_cm ** 2
    uv = uv_points(1500, 2e9)
    dx, dy, rot = 0.3 * MAS_TO_RAD, -0.2 * MAS_TO_RAD, 0.7
    vis, st = ctx.visibilities(jet.desc(), plane.desc(), nu, p, uv, rad_per_cm, jy, dx, dy, rot)
    assert vis.shape == (nu.size, uv.shape[0])
    _, _, sizes = ctx.plane_rays(plane.desc())
    sizes = sizes.reshape(plane.image_size)[0]
    across, along = pixel_centres(sizes, plane.image_size[0])
    flux_w = sizes[None, :] ** 2 * jy
    for f in range(nu.size):
        ref = direct_sum(img["I"][f] * flux_w, across, along, uv, rad_per_cm, dx, dy, rot)
        err = np.linalg.norm(vis[f] - ref) / np.linalg.norm(ref)
        assert err < 1e-6, (f, err)
        assert np.max(np.abs(vis[f] - ref)) < 1e-6 * np.max(np.abs(ref))
        # zero spacing: the total flux density of the image
        assert abs(vis[f][0] - (img["I"][f] * flux_w).sum()) < 1e-6 * abs(vis[f][0])
        # the longest baselines turn the phase across the image by tens to
        # hundreds of cycles
        assert 2e9 * np.ptp(along) * rad_per_cm > 25


def test_get_i_visibilities_drop_in(ctx):
    """pyjetshow.get_i_visibilities against the direct sum of get_i_image's
    own Jy image (the fitting loop's image -> ft step, fused)."""
    import pyjetshow

    args = (0.1, 0.1, 48, 32, 1e-2, 1e-1, 0.05, 0.1, 1.0, 500.0, 2.0, 10.0, 15.4)
    tau, img = pyjetshow.get_i_image(*args)
    uv = uv_points(600, 2e8, seed=5)
    vis = pyjetshow.get_i_visibilities(*args, uv=uv, dx=0.1, dy=0.05, rot=0.3)
    from jetshow_gb300.runtime import mas_to_pc
    pcm = mas_to_pc(0.1)
    rad_per_cm = MAS_TO_RAD / (pcm * J.pc)
    plane = J.ImagePlane((32, 48), math.log10(1e-2 * pcm * J.pc), math.log10(1e-1 * pcm * J.pc), 0.1)
    _, _, sizes = ctx.plane_rays(plane.desc())
    across, along = pixel_centres(sizes.reshape(32, 48)[0], 32)
    ref = direct_sum(img, across, along, uv, rad_per_cm, 0.1 * MAS_TO_RAD, 0.05 * MAS_TO_RAD, 0.3)
    assert np.linalg.norm(vis - ref) / np.linalg.norm(ref) < 1e-6
