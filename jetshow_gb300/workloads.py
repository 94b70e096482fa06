"""Synthetic jet workloads of the benchmark configurations.

* ``conical_c0`` -- conical jet, apex at the origin, axis +z, half-opening
  0.05 rad, LOS 0.1 rad, z = 0.1 (flat LCDM H0 = 70, Om = 0.3); helical B
  0.1 G (r/pc)^-1 with toroidal/poloidal ratio 1; n = 500 (r/pc)^-2,
  p = 2.5, gamma_min = 10; bulk Gamma = 10 along the axis; 128x128 uniform
  0.1 mas pixels at 15.4 GHz; tau then IQUV at rtol 1e-6, atol 1e-10.
* ``conical_c1`` -- the same model on a 512x1024 log-spaced plane
  (lg pixel size in mas from -3 to -1) at 8.1, 8.4, 12.1 and 15.4 GHz.
* ``parabolic_c2`` -- ParabaloidCone (r0 = 0.1 pc at 1 pc, break at 1 pc),
  LOS 0.05 rad, helical B pitch 45 deg, B0 = 1 G at 1 pc, thermal fraction
  0.1; 1024x1024 at 0.02 mas, 5 and 15.4 GHz.

Every workload returns (Jet, ImagePlane, nu[Hz, source frame], params kw).
``scale`` shrinks the image (for tests) keeping the physical extent.
"""
from __future__ import annotations

import math

import numpy as np

from . import jet as J
from .runtime import mas_to_pc

Z = 0.1
COSMO_FLAT = dict(H0=70.0, omega_M=0.3, omega_V=0.7, gamma_nu=0.0)


def pc_per_mas(z=Z):
    return mas_to_pc(z, **COSMO_FLAT)


def _lg_cm(mas, z=Z):
    return math.log10(mas * pc_per_mas(z) * J.pc)


def conical_model(half_angle=0.05, b0=0.1, n0=500.0, gamma=10.0, s=2.5, gamma_min=10.0, pitch=math.pi / 4,
                  thermal_fraction=0.0):
    geo = J.Cone((0, 0, 0), (0, 0, 1), half_angle, 100.0 * J.pc)
    return J.Jet(geo, J.ConstFlatVField(gamma), J.HelicalConicalBField(b0, 1.0, pitch, True),
                 J.BKNField(n0, 2.0, True), s=s, gamma_min=gamma_min, thermal_fraction=thermal_fraction)


TRANSFER_KW = dict(n=100, tau_max=1e4, tau_min=1e-10, tau_atol=1e-10, tau_rtol=1e-6, atol=1e-10, rtol=1e-6,
                   output="full")

# Tolerances at which the transfer of these jets is within 1e-4 of a
# converged solution (rtol 1e-10) in Stokes I wherever I > 1e-6 max(I) and
# within 1e-5 in tau.  With the configurations' atol = 1e-10 the faint,
# optically thin rays far from the core sit at the absolute-tolerance floor:
# steps grow until they straddle the narrow dip of B_perp where a ray passes
# the jet axis, the embedded error estimate misses it, and even FP64 is off
# by ~2 %.  Relative control (atol negligible) with rtol 1e-6 on IQUV and
# 1e-7 on tau keeps every sampled pixel within 3e-7 (I) and 2e-6 (tau).
ACCURATE_KW = dict(n=100, tau_max=1e4, tau_min=1e-10, tau_atol=1e-20, tau_rtol=1e-7, atol=1e-24, rtol=1e-6,
                   output="full")
# Converged reference settings (the FP64 oracle at rtol 1e-10).
CONVERGED_KW = dict(n=100, tau_max=1e4, tau_min=1e-10, tau_atol=1e-20, tau_rtol=1e-10, atol=1e-30, rtol=1e-10,
                    output="full")


def conical_c0(scale=1):
    n = max(2, 128 // scale)
    n += n % 2
    mas = 0.1 * 128 / n
    plane = J.ImagePlane((n, n), _lg_cm(mas), _lg_cm(mas), 0.1)
    nu = np.array([15.4e9]) * (1 + Z)
    return conical_model(), plane, nu, dict(TRANSFER_KW)


def conical_c1(scale=1, n_freq=4):
    na, nl = max(2, 512 // scale), max(2, 1024 // scale)
    na += na % 2
    plane = J.ImagePlane((na, nl), _lg_cm(10 ** -3), _lg_cm(10 ** -1), 0.1)
    nu = np.array([8.1e9, 8.4e9, 12.1e9, 15.4e9][:n_freq]) * (1 + Z)
    return conical_model(), plane, nu, dict(TRANSFER_KW)


def parabolic_c2(scale=1, n_freq=2):
    n = max(2, 1024 // scale)
    n += n % 2
    mas = 0.02 * 1024 / n
    geo = J.ParabaloidCone((0, 0, 0), (0, 0, 1), 0.1 * J.pc, 1.0 * J.pc, 100.0 * J.pc)
    jet = J.Jet(geo, J.ConstFlatVField(10.0), J.HelicalConicalBField(1.0, 1.0, math.pi / 4, True),
                J.BKNField(500.0, 2.0, True), s=2.5, gamma_min=10.0, thermal_fraction=0.1)
    plane = J.ImagePlane((n, n), _lg_cm(mas), _lg_cm(mas), 0.05)
    nu = np.array([5.0e9, 15.4e9][:n_freq]) * (1 + Z)
    return jet, plane, nu, dict(TRANSFER_KW)
