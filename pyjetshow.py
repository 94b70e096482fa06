"""``pyjetshow`` under the reference's own module name.

The reference builds a pybind11 module named ``pyjetshow``
(src/pyjetshow.cpp:181-201) and its fitting code imports it as
``from pyjetshow import get_i_image`` (jetmodel.py:6).  With this
repository's root on ``sys.path`` (or installed beside ``jetshow_gb300``)
that import line works unchanged and renders on the GB300:

* ``get_i_image(los_angle, redshift, number_of_pixels_along,
  number_of_pixels_across, pixel_size_mas_start, pixel_size_mas_stop,
  cone_half_angle, B_1, m, K_1, n, Gamma, nu_observed_ghz, tau_max=1e4,
  central_vfield=False) -> (tau, I_Jy)``: the reference's name, arguments,
  defaults and return value ([n_across][n_along] numpy arrays instead of
  lists of lists);
* ``get_iquv_image(...)``: the same model with the full-Stokes pass,
  returning (tau, I, Q, U, V) in Jy per pixel (new);
* ``get_i_visibilities(..., uv, dx, dy, rot)``: the visibilities of that
  image at (u, v) points, transformed on the device (JetModelZoom.ft of
  jetmodel.py:114-132; new).

There is no CPU path: the call needs the built CUDA library and a GB300.
"""
from jetshow_gb300.pyjetshow import get_i_image, get_i_visibilities, get_iquv_image

__all__ = ["get_i_image", "get_iquv_image", "get_i_visibilities"]
