"""TEST INFRASTRUCTURE: FP64 direct sum of the visibility step.

The reference transforms the rendered image with FINUFFT's type-3 NUFFT at
eps 1e-6 (JetModelZoom.ft, jetmodel.py:114-132; FINUFFT_NUNU.forward,
fourier.py:40-94):
    V(u, v) = exp(-2 pi i (u dx + v dy)) sum_j F_j exp(-2 pi i (u' x_j + v' y_j)),
    (u', v') = (u, v) @ [[cos rot, -sin rot], [sin rot, cos rot]],
with the pixel centres of JetModelZoom.calculate_grid (x = d = -pc_y across
the jet, y = r_ob along it) in radians and the flux densities F_j [Jy].
This module evaluates that sum exactly in FP64 with numpy (the value the
NUFFT approximates), for the parity tests of the device transform.
"""
import numpy as np


def pixel_centres(sizes_along, n_across):
    """Across and along centres [n_across, n_along] (cm) of a plane whose
    column j has square pixels of side sizes_along[j] (Image::Image,
    src/Image.cpp:44-185; JetModelZoom.calculate_grid): along = running sum
    minus half a size; across = +(k + 1/2) size for the upper half (rows
    counted downwards), -(k + 1/2) size for the lower half."""
    s = np.asarray(sizes_along, dtype=np.float64)
    along = np.cumsum(s) - 0.5 * s
    k = (n_across - 1) / 2.0 - np.arange(n_across)
    across = k[:, None] * s[None, :]
    return across, np.broadcast_to(along, (n_across, s.size))


def direct_sum(flux, across_cm, along_cm, uv, rad_per_cm, dx=0.0, dy=0.0, rot=0.0):
    """flux [n_pix] Jy, across/along [n_pix] cm, uv [n_uv, 2] wavelengths."""
    x = -np.asarray(across_cm, dtype=np.float64).ravel() * rad_per_cm
    y = np.asarray(along_cm, dtype=np.float64).ravel() * rad_per_cm
    f = np.asarray(flux, dtype=np.float64).ravel()
    keep = f != 0
    x, y, f = x[keep], y[keep], f[keep]
    uv = np.asarray(uv, dtype=np.float64)
    c, s = np.cos(rot), np.sin(rot)
    up = uv[:, 0] * c + uv[:, 1] * s
    vp = -uv[:, 0] * s + uv[:, 1] * c
    out = np.empty(uv.shape[0], dtype=np.complex128)
    for a in range(0, uv.shape[0], 256):
        ph = np.outer(up[a:a + 256], x) + np.outer(vp[a:a + 256], y)
        ph -= np.rint(ph)  # reduce to the fractional cycle before exp
        out[a:a + 256] = np.exp(-2j * np.pi * ph) @ f
    return out * np.exp(-2j * np.pi * (uv[:, 0] * dx + uv[:, 1] * dy))
