"""Known answers of every field law (B, N, V) of the oracle.

Each expected value is the reference's formula, restated here in numpy from
its source (the file:line of every law is cited) and evaluated at chosen
points, including the points where the reference's quirks show: atan(y/x)
for x < 0 (ToroidalBField, ForceFreeCylindricalBField), both force-free
components on sin(phi), ShearedCentralVField's acos(z + o_z / r) with z in
cm, SheathCentralVField's acos(z / r) without the origin, the composite
laws' switch on |z| with the 3-D radius inside, the parabolic flows on the
axis.  The device's FP64 laws are compared with the oracle's in the GPU
renders, so these answers pin both.  Also the first-step schedule of the
I pass (steps_schedule).
"""
import math

import numpy as np
import pytest
from scipy.special import iv

from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W

PC = 3.0856775814671913e18  # include/utils.h:20
C_CM = 29979245800.0        # include/utils.h:32

PTS = np.array([[0.3, 0.4, 2.0], [-0.5, 0.2, 1.5], [0.1, -0.7, 4.0], [-0.2, -0.3, 0.7], [0.0, 0.6, 3.0],
                [1.2, 0.05, 9.0]]) * PC


def fields(oracle, bfield=None, nfield=None, vfield=None, pts=PTS):
    jet = W.conical_model()
    if bfield is not None:
        jet.bfield = bfield
    if nfield is not None:
        jet.nfield = nfield
    if vfield is not None:
        jet.vfield = vfield
    return np.array([oracle.fields(jet.desc(), p) for p in pts])


def close(got, want):
    assert np.allclose(got, want, rtol=1e-13, atol=0.0, equal_nan=True), (got, want)


def speed(g):
    return C_CM * np.sqrt(1.0 - 1.0 / (g * g))


# ------------------------------------------------------------------- B
def test_scalar_b_laws(oracle):
    x, y, z = PTS.T
    r = np.linalg.norm(PTS, axis=1)
    # src/BField.cpp:38-41
    close(fields(oracle, J.RandomScalarBField(0.3, 1.2))[:, 0], 0.3 * (r / PC) ** -1.2)
    # src/BField.cpp:47-50
    close(fields(oracle, J.RandomScalarBFieldZ(0.3, 1.2))[:, 0], 0.3 * (np.abs(z) / PC) ** -1.2)
    # src/BField.cpp:56-64: the switch on |z| > z0, each side its own exponent
    z0 = 2.5 * PC
    want = np.where(np.abs(z) > z0, 0.3 * (np.abs(z) / PC) ** -1.7, 0.3 * (np.abs(z) / PC) ** -1.1)
    close(fields(oracle, J.CompositeRandomScalarBFieldZ(0.3, 1.1, 1.7, z0))[:, 0], want)


def test_vector_b_laws(oracle):
    x, y, z = PTS.T
    r = np.linalg.norm(PTS, axis=1)
    rc = np.hypot(x, y)
    zero = np.zeros_like(x)
    # src/BField.cpp:70-73 (the 3-D radius) and :79-82 (|z|)
    close(fields(oracle, J.ConstCylinderBField(0.2, 1.3, True))[:, :3],
          np.stack([zero, zero, 0.2 * (r / PC) ** -1.3], 1))
    close(fields(oracle, J.ConstCylinderBFieldZ(0.2, 1.3, True))[:, :3],
          np.stack([zero, zero, 0.2 * (np.abs(z) / PC) ** -1.3], 1))
    # src/BField.cpp:88-93
    b = 0.2 * (r / PC) ** -1.3
    close(fields(oracle, J.RadialConicalBField(0.2, 1.3, True))[:, :3], np.stack([b * x / r, b * y / r, b * z / r], 1))
    # src/BField.cpp:99-106: phi = atan(y / x), not atan2 (x < 0 flips B)
    fi = np.arctan(y[x != 0] / x[x != 0])
    b = 0.2 * (z[x != 0] / PC) ** -1.3
    close(fields(oracle, J.ToroidalBField(0.2, 1.3, True), pts=PTS[x != 0])[:, :3],
          np.stack([-np.sin(fi) * b, np.cos(fi) * b, np.zeros_like(b)], 1))
    # src/BField.cpp:112-117
    psi = 0.6
    close(fields(oracle, J.HelicalCylinderBField(0.2, psi, True))[:, :3],
          np.stack([0.2 * np.tan(psi * y / rc), -0.2 * np.tan(psi * x / rc), np.full_like(x, 0.2)], 1))
    # src/BField.cpp:123-131
    bz = 0.2 / (z * z / (PC * PC))
    close(fields(oracle, J.SpiralConicalBField(0.2, psi, True))[:, :3],
          np.stack([bz * (x / z + y * math.tan(psi) / PC), bz * (y / z - x * math.tan(psi) / PC), bz], 1))
    # src/BField.cpp:137-146: modified Bessel functions I0, I1 of mu, and
    # sin(phi) in both transverse components
    mu = 1.7
    fi = np.arctan(y[x != 0] / x[x != 0])
    close(fields(oracle, J.ForceFreeCylindricalBField(0.2, mu, True), pts=PTS[x != 0])[:, :3],
          np.stack([-0.2 * iv(1, mu) * np.sin(fi), 0.2 * iv(1, mu) * np.sin(fi),
                    np.full_like(fi, 0.2 * iv(0, mu))], 1))


def test_helical_conical_b(oracle):
    """The builder-defined helical conical field (no reference class):
    b0 (r/pc)^-n (sin(psi) phi_hat + cos(psi) z_hat), phi_hat = (-y, x) / r_c;
    with the atan quirk phi_hat flips for x < 0, as ToroidalBField's does."""
    x, y, z = PTS.T
    r = np.linalg.norm(PTS, axis=1)
    rc = np.hypot(x, y)
    b = 0.4 * (r / PC) ** -1.0
    psi = math.pi / 5
    for quirk in (False, True):
        s = np.where(quirk & (x < 0), -1.0, 1.0)
        want = np.stack([b * math.sin(psi) * s * -y / rc, b * math.sin(psi) * s * x / rc, b * math.cos(psi)], 1)
        close(fields(oracle, J.HelicalConicalBField(0.4, 1.0, psi, True, atan_quirk=quirk))[:, :3], want)


# ------------------------------------------------------------------- N
def test_n_laws(oracle):
    x, y, z = PTS.T
    r = np.linalg.norm(PTS, axis=1)
    close(fields(oracle, nfield=J.ConstNField(42.0, True))[:, 3], np.full_like(x, 42.0))  # src/NField.cpp:19-21
    close(fields(oracle, nfield=J.BKNField(500.0, 2.0, True))[:, 3], 500.0 * (r / PC) ** -2.0)  # :27-30
    close(fields(oracle, nfield=J.BKNFieldZ(500.0, 2.0, True))[:, 3], 500.0 * (np.abs(z) / PC) ** -2.0)  # :36-39
    # src/NField.cpp:45-53: the switch on |z|, each side a BKNField of the 3-D radius
    z0 = 2.5 * PC
    want = np.where(np.abs(z) > z0, 500.0 * (r / PC) ** -2.5, 500.0 * (r / PC) ** -1.5)
    close(fields(oracle, nfield=J.CompositeBKNField(500.0, 1.5, 2.5, z0, True))[:, 3], want)


# ------------------------------------------------------------------- V
def test_flat_v_laws(oracle):
    x, y, z = PTS.T
    rc = np.hypot(x, y)
    zero = np.zeros_like(x)
    close(fields(oracle, vfield=J.ConstFlatVField(10.0))[:, 4:], np.stack([zero, zero, speed(10.0) + zero], 1))  # :27-29
    rb = 1.5 * PC
    g = 10.0 - (10.0 - 3.0) * rc / rb                                                                           # :35-41
    close(fields(oracle, vfield=J.ShearedFlatVField(10.0, 3.0, rb))[:, 4:], np.stack([zero, zero, speed(g)], 1))
    rs = 0.5 * PC
    g = np.where(rc < rs, 12.0, 4.0)                                                                            # :47-58
    close(fields(oracle, vfield=J.SheathFlatVField(12.0, 4.0, rs))[:, 4:], np.stack([zero, zero, speed(g)], 1))


def test_central_v_laws(oracle):
    o = np.array([0.1, -0.2, 0.5]) * PC
    q = PTS + o
    r = np.linalg.norm(q, axis=1)
    # src/VField.cpp:64-71
    close(fields(oracle, vfield=J.ConstCentralVField(8.0, o))[:, 4:], speed(8.0) * q / r[:, None])
    # src/VField.cpp:93-108: theta = acos(z / r) without the origin's z
    th = np.arccos(PTS[:, 2] / r)
    g = np.where(th < 0.3, 9.0, 2.5)
    close(fields(oracle, vfield=J.SheathCentralVField(9.0, 2.5, 0.3, o))[:, 4:], speed(g)[:, None] * q / r[:, None])
    # src/VField.cpp:78-87: theta = acos(z + o_z / r) with z in cm: NaN at
    # any point of a jet; finite only within a cm of z = 0
    pts = np.array([[0.3 * PC, 0.4 * PC, 0.25], [-0.5 * PC, 0.2 * PC, -0.4]])
    o2 = np.array([0.1, -0.2, 0.0]) * PC
    q2 = pts + o2
    r2 = np.linalg.norm(q2, axis=1)
    th = np.arccos(pts[:, 2] + o2[2] / r2)
    g = 9.0 - (9.0 - 2.5) * th / 0.3
    close(fields(oracle, vfield=J.ShearedCentralVField(9.0, 2.5, 0.3, o2), pts=pts)[:, 4:],
          speed(g)[:, None] * q2 / r2[:, None])
    with np.errstate(invalid="ignore"):
        assert np.isnan(fields(oracle, vfield=J.ShearedCentralVField(9.0, 2.5, 0.3, o))[:, 4:]).all()


def parabolic_dir(v_r, Rz0, p):
    """src/VField.cpp:114-131's direction: along the paraboloid through the
    point (alpha = atan(2 pc r / r0^2)), +z on the axis."""
    x, y, z = p.T
    r = np.hypot(x, y)
    with np.errstate(divide="ignore", invalid="ignore"):
        R = np.sqrt(Rz0 * Rz0 * z / PC)
        r0 = Rz0 * r / R
        a = np.arctan(2 * PC * r / r0 / r0)
        out = np.stack([v_r * np.cos(a) * x / r, v_r * np.cos(a) * y / r, v_r * np.sin(a)], 1)
    out[r == 0] = np.stack([np.zeros_like(v_r), np.zeros_like(v_r), v_r], 1)[r == 0] if np.ndim(v_r) else [0, 0, v_r]
    return out


def test_parabolic_v_laws(oracle):
    pts = np.vstack([PTS, [[0.0, 0.0, 2.0 * PC]]])  # and a point on the axis
    x, y, z = pts.T
    r = np.hypot(x, y)
    Rz0 = 0.3 * PC
    close(fields(oracle, vfield=J.ConstParabolicVField(7.0, Rz0), pts=pts)[:, 4:],
          parabolic_dir(speed(7.0), Rz0, pts))                                                     # :114-131
    R0 = 2.0 * PC
    g = 1 + (7.0 - 1) / math.sqrt(R0) * np.sqrt(z)                                                 # :138-157
    close(fields(oracle, vfield=J.AccParabolicVField(7.0, R0, Rz0), pts=pts)[:, 4:], parabolic_dir(speed(g), Rz0, pts))
    # src/VField.cpp:171-199: the shear set at z = R0 by r / R there, (.)^0.25
    Rb = math.sqrt(Rz0 * Rz0 * R0 / PC)
    R = np.sqrt(Rz0 * Rz0 * z / PC)
    g0 = 9.0 - (9.0 - 2.0) * (Rb * r / R / Rb) ** 0.25
    g0 = np.maximum(g0, 1.0)
    g = 1 + (g0 - 1) / math.sqrt(R0) * np.sqrt(z)
    close(fields(oracle, vfield=J.ShearedAccParabolicVField(9.0, 2.0, R0, Rz0), pts=pts)[:, 4:],
          parabolic_dir(speed(g), Rz0, pts))


def test_parabolic_cone_v_laws(oracle):
    """src/VField.cpp:221-237 and :245-265: a paraboloid below z0, a cone
    above, whose origin sits on the axis where the paraboloid's tangent at
    z0 meets it (Rz0 sqrt(z0/pc) / (0.5 Rz0 (z0 pc)^-1/2) - z0)."""
    Rz0, z0 = 0.3 * PC, 2.0 * PC
    oz = Rz0 * math.sqrt(z0 / PC) / (0.5 * Rz0 * (z0 * PC) ** -0.5) - z0
    below = PTS[PTS[:, 2] <= z0]
    above = PTS[PTS[:, 2] > z0]
    # the accelerating paraboloid with R0 = z0 below, a ConstCentralVField above
    g = 1 + (6.0 - 1) / math.sqrt(z0) * np.sqrt(below[:, 2])
    close(fields(oracle, vfield=J.AccParabolicConstConeVField(6.0, Rz0, z0), pts=below)[:, 4:],
          parabolic_dir(speed(g), Rz0, below))
    q = above + [0.0, 0.0, oz]
    r = np.linalg.norm(q, axis=1)
    close(fields(oracle, vfield=J.AccParabolicConstConeVField(6.0, Rz0, z0), pts=above)[:, 4:],
          speed(6.0) * q / r[:, None])
    # the sheared versions: ShearedAccParabolicVField(R0 = z0) below,
    # ShearedCentralVField (theta atan(sqrt(Rz0^2 z0 / pc) / z0)) above, whose
    # acos(z + o_z / r) quirk makes it NaN at these points
    Rb = math.sqrt(Rz0 * Rz0 * z0 / PC)
    x, y, z = below.T
    R = np.sqrt(Rz0 * Rz0 * z / PC)
    g0 = np.maximum(9.0 - (9.0 - 2.0) * (Rb * np.hypot(x, y) / R / Rb) ** 0.25, 1.0)
    g = 1 + (g0 - 1) / math.sqrt(z0) * np.sqrt(z)
    close(fields(oracle, vfield=J.ShearedAccParabolicConstConeVField(9.0, 2.0, Rz0, z0), pts=below)[:, 4:],
          parabolic_dir(speed(g), Rz0, below))
    with np.errstate(invalid="ignore"):
        assert np.isnan(fields(oracle, vfield=J.ShearedAccParabolicConstConeVField(9.0, 2.0, Rz0, z0),
                               pts=above)[:, 4:]).all()


# ---------------------------------------------------------- steps_schedule
def test_steps_schedule(oracle):
    """src/utils.cpp:354-366 with the I pass's arguments
    (src/Observation.cpp:254-258: n, 10 n, tau_n_min 0.1, tau_n_max 100):
    n below 0.1, 10 n above 100, n + 10 n (ln tau + ln 10)^2 / (ln 100 +
    ln 10)^2 rounded up between."""
    n = 100
    for tau in (0.0, 0.05, 0.1, 0.100001, 0.5, 1.0, 3.7, 10.0, 55.0, 99.999, 100.0, 1e4):
        if tau <= 0.1:
            want = n
        elif tau >= 100.0:
            want = 10 * n
        else:
            b = -math.log(0.1)
            want = math.ceil(10 * n / (math.log(100.0) + b) ** 2 * (math.log(tau) + b) ** 2 + n)
        assert oracle.lib().jo_steps_schedule(tau, n, 10 * n) == want, tau
