"""Drop-in for the reference's ``pyjetshow`` module (src/pyjetshow.cpp:69-201).

``get_i_image`` keeps the reference's name, arguments, defaults and return
value: (tau, I in Jy per pixel) as [n_across][n_along] arrays.  The model it
builds is the reference's: Cone(0, +z, cone_half_angle, scale 100 cm),
RandomScalarBFieldZ(B_1, m), BKNFieldZ(K_1, n, plasma frame),
ConstFlat/ConstCentral VField(Gamma), s = 3.42 (src/Jet.cpp:32), WMAP9-like
cosmology of include/utils.h:172, reference tolerances.  ``get_iquv_image``
is new: the same model with the full-Stokes pass, returning
(tau, I, Q, U, V) in Jy per pixel.
"""
from __future__ import annotations

import math

import numpy as np

from . import jet as J
from .runtime import default_context, mas_to_pc


def _setup(los_angle, redshift, number_of_pixels_along, number_of_pixels_across, pixel_size_mas_start,
           pixel_size_mas_stop, cone_half_angle, B_1, m, K_1, n, Gamma, central_vfield):
    geometry = J.Cone((0., 0., 0.), (0., 0., 1.), cone_half_angle, 100)
    bfield = J.RandomScalarBFieldZ(B_1, m)
    nfield = J.BKNFieldZ(K_1, n, True)
    vfield = J.ConstCentralVField(Gamma) if central_vfield else J.ConstFlatVField(Gamma)
    jet = J.Jet(geometry, vfield, bfield, nfield, s=3.42)
    pc_in_mas = mas_to_pc(redshift)
    lg_start = math.log10(pixel_size_mas_start * pc_in_mas * J.pc)
    lg_stop = math.log10(pixel_size_mas_stop * pc_in_mas * J.pc)
    plane = J.ImagePlane((number_of_pixels_across, number_of_pixels_along), lg_start, lg_stop, los_angle)
    return jet, plane, pc_in_mas


def _jy_scale(plane, pc_in_mas, redshift, ctx):
    # I_Jy = I * Omega_pix * 1e23 / (1+z)^3 (src/pyjetshow.cpp:111-169)
    sizes = plane.getPixelSizes(ctx)
    omega = (sizes / (pc_in_mas * J.pc)) * (sizes / (pc_in_mas * J.pc)) * J.mas_to_rad * J.mas_to_rad
    return 1E-23 * (1. + redshift) * (1. + redshift) * (1. + redshift) / omega


def _run(output, los_angle, redshift, number_of_pixels_along, number_of_pixels_across, pixel_size_mas_start,
         pixel_size_mas_stop, cone_half_angle, B_1, m, K_1, n, Gamma, nu_observed_ghz, tau_max, central_vfield,
         ctx=None, **kw):
    ctx = ctx or default_context()
    jet, plane, pc_in_mas = _setup(los_angle, redshift, number_of_pixels_along, number_of_pixels_across,
                                   pixel_size_mas_start, pixel_size_mas_stop, cone_half_angle, B_1, m, K_1, n,
                                   Gamma, central_vfield)
    nu = np.atleast_1d(np.asarray(nu_observed_ghz, dtype=np.float64)) * 1E+09 * (1. + redshift)
    obs = J.Observation(jet, plane, nu)
    # src/pyjetshow.cpp:143-156: n = 100, dt_max = pc * 0.001 handed to run(),
    # which multiplies by pc once more (src/Observation.cpp:23), tau_min = 1e-10
    obs.run(100, tau_max, J.pc * 0.001, 1e-10, "adaptive", output, 2000, 0.1, tau_max, ctx=ctx, **kw)
    scales = _jy_scale(plane, pc_in_mas, redshift, ctx)
    return obs, scales


def get_i_image(los_angle, redshift, number_of_pixels_along, number_of_pixels_across, pixel_size_mas_start,
                pixel_size_mas_stop, cone_half_angle, B_1, m, K_1, n, Gamma, nu_observed_ghz, tau_max=10000.,
                central_vfield=False, **kw):
    """Stokes I image with a tangled B field: returns (tau, I_Jy)."""
    obs, scales = _run("I", los_angle, redshift, number_of_pixels_along, number_of_pixels_across,
                       pixel_size_mas_start, pixel_size_mas_stop, cone_half_angle, B_1, m, K_1, n, Gamma,
                       nu_observed_ghz, tau_max, central_vfield, **kw)
    return obs.getImage("tau"), obs.getImage("I") / scales


def get_iquv_image(los_angle, redshift, number_of_pixels_along, number_of_pixels_across, pixel_size_mas_start,
                   pixel_size_mas_stop, cone_half_angle, B_1, m, K_1, n, Gamma, nu_observed_ghz, tau_max=10000.,
                   central_vfield=False, **kw):
    """Full-Stokes image of the same model: returns (tau, I, Q, U, V) in Jy.
    With the tangled (scalar) field Q = U = V = 0."""
    obs, scales = _run("full", los_angle, redshift, number_of_pixels_along, number_of_pixels_across,
                       pixel_size_mas_start, pixel_size_mas_stop, cone_half_angle, B_1, m, K_1, n, Gamma,
                       nu_observed_ghz, tau_max, central_vfield, **kw)
    return (obs.getImage("tau"),) + tuple(obs.getImage(k) / scales for k in ("I", "Q", "U", "V"))


MAS_TO_RAD = 4.84813681109536e-09


def get_i_visibilities(los_angle, redshift, number_of_pixels_along, number_of_pixels_across, pixel_size_mas_start,
                       pixel_size_mas_stop, cone_half_angle, B_1, m, K_1, n, Gamma, nu_observed_ghz, uv, dx=0.0,
                       dy=0.0, rot=0.0, tau_max=10000., central_vfield=False, pc_per_mas_uv=None, ctx=None, **kw):
    """Visibilities [Jy] of the get_i_image model at ``uv`` [n_uv, 2]
    (wavelengths), as JetModelZoom.ft computes them: shift by (dx, dy) mas,
    (u, v) rotated by ``rot``, pixel centres at the image's own coordinates
    (across with the "d = -pc_y" sign), flux densities in Jy per pixel.
    ``pc_per_mas_uv`` sets the angular scale of the pixel coordinates (the
    fitting code takes it from its own cosmology); by default the binding's
    mas_to_pc(redshift).  Returns complex [n_uv] (one frequency) or
    [n_nu, n_uv]."""
    ctx = ctx or default_context()
    jet, plane, pc_in_mas = _setup(los_angle, redshift, number_of_pixels_along, number_of_pixels_across,
                                   pixel_size_mas_start, pixel_size_mas_stop, cone_half_angle, B_1, m, K_1, n,
                                   Gamma, central_vfield)
    nu = np.atleast_1d(np.asarray(nu_observed_ghz, dtype=np.float64)) * 1E+09 * (1. + redshift)
    p = J.make_params(n=100, tau_max=tau_max, dt_max=J.pc * 0.001 * J.pc, tau_min=1e-10, output="I", **kw)
    pcm_uv = pc_in_mas if pc_per_mas_uv is None else float(pc_per_mas_uv)
    jy = 1e23 / (1. + redshift) ** 3 * (MAS_TO_RAD / (pc_in_mas * J.pc)) ** 2
    vis, _ = ctx.visibilities(jet.desc(), plane.desc(), nu, p, uv, MAS_TO_RAD / (pcm_uv * J.pc), jy,
                              dx * MAS_TO_RAD, dy * MAS_TO_RAD, rot)
    return vis[0] if np.ndim(nu_observed_ghz) == 0 else vis
