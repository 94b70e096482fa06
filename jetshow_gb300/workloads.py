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
``scale`` shrinks the image (for tests) keeping the physical extent; ``pcm``
(parsecs per mas at z = 0.1 in the flat cosmology) is computed with the
library's ``jsh_mas_to_pc`` unless the caller passes it (the CPU reference
arm of the benchmark passes the oracle's value, which is bitwise the same).
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


def _lg_cm(mas, z=Z, pcm=None):
    return math.log10(mas * (pcm if pcm is not None else pc_per_mas(z)) * J.pc)


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
# 1e-7 on tau keeps every sampled FP64 pixel within 3e-7 (I) and 2e-6 (tau);
# the FP32-stage path needs 5e-8 on tau to keep its worst sampled ray below
# 4e-6 (at 1e-7 one far ray reaches 1.1e-5), for 7 % more work.
ACCURATE_KW = dict(n=100, tau_max=1e4, tau_min=1e-10, tau_atol=1e-20, tau_rtol=5e-8, atol=1e-24, rtol=1e-6,
                   output="full")
# I-only output: the step control sees only I, and rtol 1e-6 leaves FP64 up
# to 3.6e-4 off the converged I on the conical jet; rtol 1e-7 gives 3.6e-6
# for 9 % more evaluations.
ACCURATE_I_KW = dict(ACCURATE_KW, rtol=1e-7, output="I")
# Gridded fields: the interpolated fields have kinks at every triangle edge
# and the adaptive steps converge slowly; on the simulation-grid jet FP64 is
# 2.2e-4 (tau) / 1.3e-4 (I) off a converged solution at ACCURATE_KW and
# 1.8e-5 / 1.7e-5 at these settings.
GRID_KW = dict(ACCURATE_KW, tau_rtol=1e-9, rtol=1e-8)
# Gridded fields, two implementations of the FP64 algorithm compared with
# each other: a last-bit difference anywhere (an fma contraction, a libm
# ulp) moves the adaptive steps across the interpolant's kinks and, at
# GRID_KW, the two images by up to 2.3e-5 in tau (measured with the oracle
# against a perturbed copy of itself); at these tolerances by 1e-6.
GRID_TIGHT_KW = dict(ACCURATE_KW, tau_rtol=1e-11, rtol=1e-10)
# Gridded fields, mixed precision: the tau pass's steps limited to 0.001 pc
# (a fifth of a triangle of the 200k-point grid) so that every kink is
# resolved, and IQUV at rtol 1e-8; measured against the oracle at tau rtol
# 1e-12 on the simulation-grid jet: tau 7.1e-6, I 5.8e-6, Q/U/V 2.5e-6 of
# max I (at ACCURATE_KW: 1.3e-4 / 1.6e-4 / 9.9e-5), for 3.1x the work.
GRID_MIXED_KW = dict(ACCURATE_KW, dt_max=0.001 * J.pc, rtol=1e-8)
# Converged reference settings (the FP64 oracle at rtol 1e-10).
CONVERGED_KW = dict(n=100, tau_max=1e4, tau_min=1e-10, tau_atol=1e-20, tau_rtol=1e-10, atol=1e-30, rtol=1e-10,
                    output="full")
# ... and for gridded fields, whose kinks converge slowly (rtol 1e-10 and
# 1e-12 differ by 4.9e-6 in tau there)
GRID_CONVERGED_KW = dict(CONVERGED_KW, tau_rtol=1e-12)


def conical_c0(scale=1, pcm=None):
    n = max(2, 128 // scale)
    n += n % 2
    mas = 0.1 * 128 / n
    plane = J.ImagePlane((n, n), _lg_cm(mas, pcm=pcm), _lg_cm(mas, pcm=pcm), 0.1)
    nu = np.array([15.4e9]) * (1 + Z)
    return conical_model(), plane, nu, dict(TRANSFER_KW)


def conical_c1(scale=1, n_freq=4, pcm=None):
    na, nl = max(2, 512 // scale), max(2, 1024 // scale)
    na += na % 2
    plane = J.ImagePlane((na, nl), _lg_cm(10 ** -3, pcm=pcm), _lg_cm(10 ** -1, pcm=pcm), 0.1)
    nu = np.array([8.1e9, 8.4e9, 12.1e9, 15.4e9][:n_freq]) * (1 + Z)
    return conical_model(), plane, nu, dict(TRANSFER_KW)


def parabolic_c2(scale=1, n_freq=2, pcm=None):
    n = max(2, 1024 // scale)
    n += n % 2
    mas = 0.02 * 1024 / n
    geo = J.ParabaloidCone((0, 0, 0), (0, 0, 1), 0.1 * J.pc, 1.0 * J.pc, 100.0 * J.pc)
    jet = J.Jet(geo, J.ConstFlatVField(10.0), J.HelicalConicalBField(1.0, 1.0, math.pi / 4, True),
                J.BKNField(500.0, 2.0, True), s=2.5, gamma_min=10.0, thermal_fraction=0.1)
    plane = J.ImagePlane((n, n), _lg_cm(mas, pcm=pcm), _lg_cm(mas, pcm=pcm), 0.05)
    nu = np.array([5.0e9, 15.4e9][:n_freq]) * (1 + Z)
    return jet, plane, nu, dict(TRANSFER_KW)


# ----------------------------------------------------------------- C3
def scrambled_sobol2(n: int, seed: int = 0, bits: int = 30) -> np.ndarray:
    """n points of the 2-D Sobol sequence (dimension 1: van der Corput;
    dimension 2: primitive polynomial x + 1, m_1 = 1) with Matousek's
    random linear scramble and a random digital shift, both drawn from
    ``seed``.  Returns float64 [n, 2] in [0, 1)."""
    rng = np.random.default_rng(seed)
    idx = np.arange(n, dtype=np.uint64)
    # direction numbers v_k = m_k 2^(bits - k), k = 1..bits
    m = [1]
    for _ in range(1, bits):
        m.append((2 * m[-1]) ^ m[-1])
    dirs = [[1 << (bits - k) for k in range(1, bits + 1)], [m[k - 1] << (bits - k) for k in range(1, bits + 1)]]
    out = np.empty((n, 2))
    for d in range(2):
        x = np.zeros(n, dtype=np.uint64)
        for k in range(bits):
            x ^= ((idx >> np.uint64(k)) & np.uint64(1)) * np.uint64(dirs[d][k])
        # linear scramble: output bit j (from the most significant) is the
        # parity of input bits 0..j under a random lower-triangular matrix
        # with unit diagonal; then a random digital shift
        y = np.zeros(n, dtype=np.uint64)
        for j in range(bits):
            row = rng.integers(0, 2, size=j + 1)
            row[j] = 1
            mask = 0
            for i in range(j + 1):
                if row[i]:
                    mask |= 1 << (bits - 1 - i)
            p = x & np.uint64(mask)
            for s in (32, 16, 8, 4, 2, 1):
                p ^= p >> np.uint64(s)
            y |= (p & np.uint64(1)) << np.uint64(bits - 1 - j)
        y ^= np.uint64(int(rng.integers(0, 1 << bits)))
        out[:, d] = y.astype(np.float64) / float(1 << bits)
    return out


def gaussian_random_field(z_max=20.0, r_max=0.5, step=0.0125, corr=0.05, seed=1):
    """Unit-variance Gaussian random field on a lattice of `step` pc over
    [0, z_max] x [0, r_max]: white noise (seeded) convolved with a Gaussian
    kernel of width corr / sqrt(2), so that the field's correlation is
    exp(-d^2 / (2 corr^2)).  Returns (lattice values [nz, nr], step)."""
    rng = np.random.default_rng(seed)
    sk = corr / math.sqrt(2.0) / step  # kernel width in lattice steps
    half = int(math.ceil(4 * sk))
    ker = np.exp(-0.5 * (np.arange(-half, half + 1) / sk) ** 2)
    ker /= np.sqrt(np.sum(ker ** 2))
    nz, nr = int(round(z_max / step)) + 1, int(round(r_max / step)) + 1
    noise = rng.standard_normal((nz + 2 * half, nr + 2 * half))
    g = np.apply_along_axis(lambda v: np.convolve(v, ker, mode="valid"), 0, noise)
    g = np.apply_along_axis(lambda v: np.convolve(v, ker, mode="valid"), 1, g)
    return g, step


def bilinear(lattice, step, z, r):
    fz, fr = z / step, r / step
    i = np.clip(np.floor(fz).astype(int), 0, lattice.shape[0] - 2)
    j = np.clip(np.floor(fr).astype(int), 0, lattice.shape[1] - 2)
    tz, tr = fz - i, fr - j
    return ((1 - tz) * (1 - tr) * lattice[i, j] + tz * (1 - tr) * lattice[i + 1, j] +
            (1 - tz) * tr * lattice[i, j + 1] + tz * tr * lattice[i + 1, j + 1])


C3_FIELDS = ("B_p", "B_phi", "n", "Gamma")


def simulation_grid_c3(n_points=200_000, sigma=0.3):
    """The C3 simulation grid: scrambled Sobol points (seed 0) over
    z in [0, 20] pc, r in [0, 0.5] pc, and the rectangle's edges every
    0.0125 pc; values B_p, B_phi, n, Gamma of the
    conical jet's laws (B = 0.1 G (R/pc)^-1 split equally poloidal /
    toroidal, n = 500 (R/pc)^-2, Gamma = 10; R = sqrt(z^2 + r^2), at least
    0.005 pc) times
    exp(sigma g) with g the seeded Gaussian random field (correlation
    0.05 pc), FP32.  Returns (xy [n, 2] float64 (z, r) pc, values [n, 4]
    float32)."""
    u = scrambled_sobol2(n_points, seed=0)
    # plus the domain's edges every 0.0125 pc, so that the hull is the whole
    # rectangle (the jet axis r = 0 included)
    ez = np.linspace(0.0, 20.0, 1601)
    er = np.linspace(0.0, 0.5, 41)[1:-1]
    z = np.concatenate([20.0 * u[:, 0], ez, ez, np.zeros(er.size), np.full(er.size, 20.0)])
    r = np.concatenate([0.5 * u[:, 1], np.zeros(ez.size), np.full(ez.size, 0.5), er, er])
    lat, step = gaussian_random_field()
    f = np.exp(sigma * bilinear(lat, step, z, r))
    R = np.maximum(np.hypot(z, r), 0.005)  # the laws are singular at the apex
    b = 0.1 * (1.0 / R) / math.sqrt(2.0)
    vals = np.column_stack([b * f, b * f, 500.0 * R ** -2 * f, 10.0 * f]).astype(np.float32)
    return np.column_stack([z, r]), vals


def simulation_c3(grid_id: int, scale=1):
    """C3 render on an uploaded C3 grid: Cone (half-angle 0.05) as the
    envelope, every field from the grid (nan_value outside its hull:
    B = n = 0, Gamma = 1), LOS 0.1 rad, 512x512 uniform pixels of
    0.0005 mas, 15.4 GHz.  A ray through the cone at height z spans
    z/1.5 .. 2z (LOS 0.1, half-angle 0.05); the 0.128 mas half-extent along
    the jet keeps every ray below z = 9.4 pc, where the cone (r <= 0.47 pc)
    is inside the grid, so no ray meets the jump to nan_value at the hull."""
    n = max(2, 512 // scale)
    n += n % 2
    mas = 0.0005 * 512 / n
    geo = J.Cone((0, 0, 0), (0, 0, 1), 0.05, 100.0 * J.pc)
    jet = J.Jet(geo, J.SimulationVField(grid_id, 3), J.SimulationBField(grid_id, 0, 1, True),
                J.SimulationNField(grid_id, 2, True), s=2.5, gamma_min=10.0)
    plane = J.ImagePlane((n, n), _lg_cm(mas), _lg_cm(mas), 0.1)
    nu = np.array([15.4e9]) * (1 + Z)
    return jet, plane, nu, dict(TRANSFER_KW)
