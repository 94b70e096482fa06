"""Host-side mirror of jetshow's model classes.

The classes keep the reference constructors (names, argument order and
meaning) and compile to the C-ABI descriptors of ``include/jetshow_capi.h``:

* geometry: ``Cone`` (include/Cone.h:14-15), ``Cylinder`` (include/Cylinder.h:14-15),
  ``Parabaloid`` (include/Parabaloid.h:18-19), ``ParabaloidCone`` (include/ParabaloidCone.h:19-20),
  ``SimulationGeometry`` (include/Geometry.h:58-65);
* fields: include/BField.h:36-208, include/NField.h:10-69, include/VField.h:11-185;
* ``Jet`` (include/Jet.h:11-61), ``ImagePlane`` (include/ImagePlane.h:22-23),
  ``Observation`` (include/Observation.h:12-24).

``Observation.run`` renders on the GPU through ``jsh_observation_run``;
there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _capi as A
from .runtime import default_context

# Constants of include/utils.h:17-36
mas_to_rad = 4.84813681109536e-09
rad_to_mas = 206264806.24709633
pc = 3.0856775814671913e+18
m_e = 9.10938356e-28
q_e = 4.80320467299766e-10
c = 29979245800.0
to_jy = 1E+23


def _v3(v) -> tuple:
    a = tuple(float(x) for x in v)
    if len(a) != 3:
        raise ValueError("expected a 3-vector")
    return a


# ------------------------------------------------------------- geometry
class _Geometry:
    def desc(self) -> A.GeometryDesc:
        raise NotImplementedError


class Cone(_Geometry):
    """Cone(origin, direction, angle, scale) -- src/Cone.cpp:16-25."""

    def __init__(self, origin, direction, angle, scale):
        self.origin, self.direction = _v3(origin), _v3(direction)
        self.angle, self.big_scale = float(angle), float(scale)

    def desc(self):
        return A.GeometryDesc(kind=A.GEO_CONE, origin=self.origin, direction=self.direction,
                              angle=self.angle, big_scale=self.big_scale)


class Cylinder(_Geometry):
    """Cylinder(origin, direction, r) -- src/Cylinder.cpp:9-15."""

    def __init__(self, origin, direction, r):
        self.origin, self.direction, self.r = _v3(origin), _v3(direction), float(r)

    def desc(self):
        return A.GeometryDesc(kind=A.GEO_CYLINDER, origin=self.origin, direction=self.direction,
                              r=self.r, big_scale=100.0 * self.r)


class Parabaloid(_Geometry):
    """Parabaloid(origin, direction, r0, big_scale) -- src/Parabaloid.cpp:11-17."""

    def __init__(self, origin, direction, r0, big_scale):
        self.origin, self.direction = _v3(origin), _v3(direction)
        self.r0, self.big_scale = float(r0), float(big_scale)

    def desc(self):
        return A.GeometryDesc(kind=A.GEO_PARABALOID, origin=self.origin, direction=self.direction,
                              r0=self.r0, big_scale=self.big_scale)


class ParabaloidCone(_Geometry):
    """ParabaloidCone(origin, direction, r0, z0, scale) -- src/ParabaloidCone.cpp:12-18."""

    def __init__(self, origin, direction, r0, z0, scale):
        self.origin, self.direction = _v3(origin), _v3(direction)
        self.r0, self.z0, self.big_scale = float(r0), float(z0), float(scale)

    def desc(self):
        return A.GeometryDesc(kind=A.GEO_PARABALOID_CONE, origin=self.origin, direction=self.direction,
                              r0=self.r0, z0=self.z0, big_scale=self.big_scale)


class SimulationGeometry(_Geometry):
    """SimulationGeometry(tree) -- src/Geometry.cpp:92-132: the convex hull of
    a simulation's (z, r) points revolved about the jet axis (the reference
    builds ``tree`` from the points at 36 azimuths, src/main.cpp:880-897).
    ``hull`` is the id returned by ``Context.hull_upload(zr, n_circle)``."""

    def __init__(self, hull):
        self.hull = int(hull)

    def desc(self):
        return A.GeometryDesc(kind=A.GEO_SIMULATION, hull_id=self.hull, direction=(0.0, 0.0, 1.0))


# --------------------------------------------------------------- fields
class _Field:
    kind = 0
    in_plasma_frame = True

    def __init__(self, *params, in_plasma_frame=True):
        self.params = [float(p) for p in params]
        self.in_plasma_frame = bool(in_plasma_frame)

    def desc(self) -> A.FieldDesc:
        p = (C.c_double * 8)(*(self.params + [0.0] * (8 - len(self.params))))
        return A.FieldDesc(kind=self.kind, in_plasma_frame=int(self.in_plasma_frame), p=p)


class RandomScalarBField(_Field):
    """b_0 (|x|/pc)^-m_b (src/BField.cpp:35-41)."""
    kind = A.B_RANDOM_SCALAR

    def __init__(self, b_0, m_b):
        super().__init__(b_0, m_b)


class RandomScalarBFieldZ(_Field):
    """b_0 (|z|/pc)^-m_b (src/BField.cpp:44-50)."""
    kind = A.B_RANDOM_SCALAR_Z

    def __init__(self, b_0, m_b):
        super().__init__(b_0, m_b)


class CompositeRandomScalarBFieldZ(_Field):
    kind = A.B_COMPOSITE_RANDOM_SCALAR_Z

    def __init__(self, b_0, m_b_inner, m_b_outer, z0):
        super().__init__(b_0, m_b_inner, m_b_outer, z0)


class ConstCylinderBField(_Field):
    kind = A.B_CONST_CYLINDER

    def __init__(self, b_0, n_b, in_plasma_frame):
        super().__init__(b_0, n_b, in_plasma_frame=in_plasma_frame)


class ConstCylinderBFieldZ(_Field):
    kind = A.B_CONST_CYLINDER_Z

    def __init__(self, b_0, n_b, in_plasma_frame):
        super().__init__(b_0, n_b, in_plasma_frame=in_plasma_frame)


class RadialConicalBField(_Field):
    kind = A.B_RADIAL_CONICAL

    def __init__(self, b_0, n_b, in_plasma_frame):
        super().__init__(b_0, n_b, in_plasma_frame=in_plasma_frame)


class ToroidalBField(_Field):
    """(-sin phi, cos phi, 0) b_0 (z/pc)^-n_b with phi = atan(y/x) (src/BField.cpp:96-106)."""
    kind = A.B_TOROIDAL

    def __init__(self, b_0, n_b, in_plasma_frame):
        super().__init__(b_0, n_b, in_plasma_frame=in_plasma_frame)


class HelicalCylinderBField(_Field):
    kind = A.B_HELICAL_CYLINDER

    def __init__(self, b_0, pitch_angle, in_plasma_frame):
        super().__init__(b_0, pitch_angle, in_plasma_frame=in_plasma_frame)


class SpiralConicalBField(_Field):
    kind = A.B_SPIRAL_CONICAL

    def __init__(self, b_0, pitch_angle, in_plasma_frame):
        super().__init__(b_0, pitch_angle, in_plasma_frame=in_plasma_frame)


class ForceFreeCylindricalBField(_Field):
    kind = A.B_FORCE_FREE_CYLINDRICAL

    def __init__(self, b_0, mu, in_plasma_frame):
        super().__init__(b_0, mu, in_plasma_frame=in_plasma_frame)


class HelicalConicalBField(_Field):
    """Builder-defined helical field of a conical jet (no reference class):
    B = b_0 (|x|/pc)^-n_b (sin(pitch) phi_hat + cos(pitch) z_hat).
    ``atan_quirk`` reproduces ToroidalBField's phi = atan(y/x) sign flip."""
    kind = A.B_HELICAL_CONICAL

    def __init__(self, b_0, n_b, pitch_angle, in_plasma_frame=True, atan_quirk=False):
        super().__init__(b_0, n_b, pitch_angle, 1.0 if atan_quirk else 0.0, in_plasma_frame=in_plasma_frame)


class SimulationBField(_Field):
    """B from an uploaded (z, r) grid: fields ``field_p`` (poloidal) and
    ``field_phi`` (toroidal) (src/BField.cpp:196-207)."""
    kind = A.B_SIMULATION

    def __init__(self, grid_id, field_p, field_phi, in_plasma_frame=True):
        super().__init__(grid_id, field_p, field_phi, in_plasma_frame=in_plasma_frame)


class RandomVectorBField:
    """RandomVectorBField(bfield, rnd_fraction) -- src/BField.cpp:149-161:
    B + rnd_fraction |B| n with n a random unit vector; the wrapper's field
    is taken in the plasma frame (the reference constructs it
    VectorBField(true)).  Use one of the two kinds below."""
    kind_random = A.RND_NONE

    def __init__(self, bfield, rnd_fraction):
        if getattr(bfield, "kind", None) in A.SCALAR_B_KINDS:
            raise ValueError("RandomVectorBField wraps a vector B field")
        self.bfield, self.rnd_fraction = bfield, float(rnd_fraction)

    def desc(self) -> A.FieldDesc:
        return self.bfield.desc()

    def random_desc(self) -> A.RandomDesc:
        return A.RandomDesc(kind=self.kind_random, fraction=self.rnd_fraction)


class CellsRandomVectorBField(RandomVectorBField):
    """CellsRandomVectorBField(cells, bfield, rnd_fraction) --
    src/BField.cpp:164-172: n is the direction of the cell nearest to the
    point.  ``cells``: an uploaded RandomCells (or its cell-set id)."""
    kind_random = A.RND_CELLS

    def __init__(self, cells, bfield, rnd_fraction):
        super().__init__(bfield, rnd_fraction)
        self.cells = cells

    def random_desc(self) -> A.RandomDesc:
        cid = self.cells if isinstance(self.cells, int) else self.cells.id
        if cid is None:
            raise RuntimeError("upload the cells first (RandomCells.upload)")
        return A.RandomDesc(kind=self.kind_random, cells_id=int(cid), fraction=self.rnd_fraction)


class PointsRandomVectorBField(RandomVectorBField):
    """PointsRandomVectorBField(bfield, rnd_fraction, seed) --
    src/BField.cpp:175-193: a fresh random direction at every evaluation,
    drawn here from a counter-based stream keyed by (seed, pixel, frequency,
    evaluation index) instead of the reference's per-thread generators."""
    kind_random = A.RND_POINTS

    def __init__(self, bfield, rnd_fraction, seed=0):
        super().__init__(bfield, rnd_fraction)
        self.seed = int(seed)

    def random_desc(self) -> A.RandomDesc:
        return A.RandomDesc(kind=self.kind_random, fraction=self.rnd_fraction, seed=self.seed)


class RandomCellsInSphere:
    """RandomCellsInSphere(N, n_exponent, seed) -- src/Cells.cpp:24-47:
    ``setGeometry(r_max, theta_max, r_min, theta_min)`` then ``create()``
    draws N cell points (generate_random_points_sphere, src/utils.cpp:267-312)
    and directions with the counter-based generator on the host
    (jsh_cells_generate); ``upload(ctx)`` puts them on the device."""

    def __init__(self, N, n_exponent, seed=0):
        self.n, self.exponent, self.seed = int(N), float(n_exponent), int(seed)
        self.r_max = self.theta_max = self.r_min = self.theta_min = 0.0
        self.points = self.directions = None
        self.id = None

    def setGeometry(self, coord1_max, coord2_max, coord1_min=0.0, coord2_min=0.0):
        self.r_max, self.theta_max, self.r_min, self.theta_min = (float(coord1_max), float(coord2_max),
                                                                  float(coord1_min), float(coord2_min))

    def create(self):
        from .runtime import cells_generate
        self.points, self.directions = cells_generate(self.n, self.r_min, self.r_max, self.theta_max,
                                                      self.exponent, self.seed)
        return self

    def getCells(self):
        return self.points

    def upload(self, ctx=None):
        if self.points is None:
            self.create()
        self.id = (ctx or default_context()).cells_upload(self.points, self.directions)
        return self.id


class ConstNField(_Field):
    kind = A.N_CONST

    def __init__(self, n, in_plasma_frame):
        super().__init__(n, in_plasma_frame=in_plasma_frame)


class BKNField(_Field):
    """n_0 (|x|/pc)^-n_n (src/NField.cpp:21-30)."""
    kind = A.N_BK

    def __init__(self, n_0, n_n, in_plasma_frame):
        super().__init__(n_0, n_n, in_plasma_frame=in_plasma_frame)


class BKNFieldZ(_Field):
    """n_0 (|z|/pc)^-n_n (src/NField.cpp:33-39)."""
    kind = A.N_BKZ

    def __init__(self, n_0, n_n, in_plasma_frame):
        super().__init__(n_0, n_n, in_plasma_frame=in_plasma_frame)


class CompositeBKNField(_Field):
    kind = A.N_COMPOSITE_BK

    def __init__(self, n_0, n_n_inner, n_n_outer, z0, in_plasma_frame):
        super().__init__(n_0, n_n_inner, n_n_outer, z0, in_plasma_frame=in_plasma_frame)


class SimulationNField(_Field):
    kind = A.N_SIMULATION

    def __init__(self, grid_id, field, in_plasma_frame=True):
        super().__init__(grid_id, field, in_plasma_frame=in_plasma_frame)


class ConstFlatVField(_Field):
    """(0, 0, c sqrt(1 - 1/Gamma^2)) (src/VField.cpp:25-29)."""
    kind = A.V_CONST_FLAT

    def __init__(self, gamma):
        super().__init__(gamma)


class ShearedFlatVField(_Field):
    kind = A.V_SHEARED_FLAT

    def __init__(self, gamma_axis, gamma_border, r):
        super().__init__(gamma_axis, gamma_border, r)


class SheathFlatVField(_Field):
    kind = A.V_SHEATH_FLAT

    def __init__(self, gamma_spine, gamma_sheath, r_sheath):
        super().__init__(gamma_spine, gamma_sheath, r_sheath)


class ConstCentralVField(_Field):
    kind = A.V_CONST_CENTRAL

    def __init__(self, gamma, origin=(0.0, 0.0, 0.0)):
        super().__init__(gamma, *_v3(origin))


class ShearedCentralVField(_Field):
    kind = A.V_SHEARED_CENTRAL

    def __init__(self, gamma_axis, gamma_border, theta, origin=(0.0, 0.0, 0.0)):
        super().__init__(gamma_axis, gamma_border, theta, *_v3(origin))


class SheathCentralVField(_Field):
    kind = A.V_SHEATH_CENTRAL

    def __init__(self, gamma_spine, gamma_sheath, theta_sheath, origin=(0.0, 0.0, 0.0)):
        super().__init__(gamma_spine, gamma_sheath, theta_sheath, *_v3(origin))


class ConstParabolicVField(_Field):
    kind = A.V_CONST_PARABOLIC

    def __init__(self, gamma, Rz0):
        super().__init__(gamma, Rz0)


class AccParabolicVField(_Field):
    kind = A.V_ACC_PARABOLIC

    def __init__(self, gamma0, R0, Rz0):
        super().__init__(gamma0, R0, Rz0)


class ShearedAccParabolicVField(_Field):
    kind = A.V_SHEARED_ACC_PARABOLIC

    def __init__(self, gamma_axis0, gamma_border0, R0, Rz0):
        super().__init__(gamma_axis0, gamma_border0, R0, Rz0)


class AccParabolicConstConeVField(_Field):
    kind = A.V_ACC_PARABOLIC_CONST_CONE

    def __init__(self, gamma0, Rz0, z0):
        super().__init__(gamma0, Rz0, z0)


class ShearedAccParabolicConstConeVField(_Field):
    kind = A.V_SHEARED_ACC_PARABOLIC_CONST_CONE

    def __init__(self, gamma_axis0, gamma_border0, Rz0, z0):
        super().__init__(gamma_axis0, gamma_border0, Rz0, z0)


class SimulationVField(_Field):
    kind = A.V_SIMULATION

    def __init__(self, grid_id, field):
        super().__init__(grid_id, field)


# ------------------------------------------------------------------ Jet
class Jet:
    """Jet(geometry, vfield, bfield, nfield) -- src/Jet.cpp:5-11.

    ``s`` is the power-law index of the coefficients (the reference
    hard-codes 3.42 in Jet::getKI / getEtaI, src/Jet.cpp:32, :234);
    ``gamma_min`` enters k_F_r and k_C_r; ``thermal_fraction`` adds cold
    k_F_c / k_C_c terms of n_th = fraction * n (builder-defined)."""

    def __init__(self, geometry, vfield, bfield, nfield, s=3.42, gamma_min=100.0, thermal_fraction=0.0):
        self.geometry, self.vfield, self.bfield, self.nfield = geometry, vfield, bfield, nfield
        self.s, self.gamma_min, self.thermal_fraction = float(s), float(gamma_min), float(thermal_fraction)

    def desc(self) -> A.ModelDesc:
        rnd = self.bfield.random_desc() if hasattr(self.bfield, "random_desc") else A.RandomDesc()
        return A.ModelDesc(geometry=self.geometry.desc(), bfield=self.bfield.desc(),
                           nfield=self.nfield.desc(), vfield=self.vfield.desc(), s=self.s,
                           gamma_min=self.gamma_min, thermal_fraction=self.thermal_fraction, random=rnd)

    def hit(self, origins, directions, ctx=None):
        """Jet::hit for arrays of rays; returns (n_seg, seg[n, 2, 2, 3], status)."""
        return (ctx or default_context()).hit_rays(self.desc(), origins, directions)


class ImagePlane:
    """ImagePlane(image_size=(n_across, n_along), lg_pixel_size_start_cm,
    lg_pixel_size_stop_cm, los_angle) -- src/ImagePlane.cpp:11-33."""

    def __init__(self, image_size, pixel_size_start, pixel_size_stop, los_angle):
        self.image_size = (int(image_size[0]), int(image_size[1]))
        self.lg_start, self.lg_stop, self.los_angle = float(pixel_size_start), float(pixel_size_stop), float(los_angle)

    def desc(self) -> A.PlaneDesc:
        return A.PlaneDesc(n_across=self.image_size[0], n_along=self.image_size[1],
                           lg_pixel_size_start_cm=self.lg_start, lg_pixel_size_stop_cm=self.lg_stop,
                           los_angle=self.los_angle)

    def getRays(self, ctx=None):
        """(origins[n_across*n_along, 3], direction[3]) generated on the device."""
        o, d, _ = (ctx or default_context()).plane_rays(self.desc())
        return o, d

    def getPixelSizes(self, ctx=None):
        _, _, s = (ctx or default_context()).plane_rays(self.desc())
        return s.reshape(self.image_size)


class Observation:
    """Observation(jet, imagePlane, nu) -- src/Observation.cpp:12-17.

    ``nu`` may be a scalar or a sequence of frequencies [Hz]; all are
    rendered in one device pass.  ``run`` keeps the reference signature
    (src/Observation.cpp:20-22): ``dt_max`` is in pc as there, and
    ``integration_type``, ``n_max``, ``tau_n_min``, ``tau_n_max`` are
    accepted and unused as in the reference.  ``output_type`` "full" now
    integrates IQUV (the reference's full-Stokes pass is commented out)."""

    def __init__(self, jet: Jet, imagePlane: ImagePlane, nu):
        self.jet, self.imagePlane = jet, imagePlane
        self.nu = np.atleast_1d(np.asarray(nu, dtype=np.float64))
        self._images = None
        self.stats = None

    def run(self, n, tau_max, dt_max, tau_min, integration_type="adaptive", output_type="I", n_max=0,
            tau_n_min=0.1, tau_n_max=100.0, *, precision="fp64", schedule="static", tau_atol=1E-7,
            tau_rtol=1E-14, atol=1E-9, rtol=1E-9, ctx=None, **kw):
        p = make_params(n=n, tau_max=tau_max, dt_max=dt_max * pc, tau_min=tau_min, output=output_type,
                        precision=precision, schedule=schedule, tau_atol=tau_atol, tau_rtol=tau_rtol,
                        atol=atol, rtol=rtol, **kw)
        self._images, self.stats = (ctx or default_context()).render(self.jet.desc(), self.imagePlane.desc(),
                                                                     self.nu, p)
        return self

    def run_stripe(self, n, tau_max, tau_min=0.0, *, freq_index: int = 0, ctx=None):
        """Observation::run_stripe (src/Observation.cpp:310-347): tau only,
        along half of the central row, constant-step RK4 (``tau_min`` is
        accepted and unused, as in the reference)."""
        self._stripe = (ctx or default_context()).stripe(self.jet.desc(), self.imagePlane.desc(),
                                                         float(self.nu[freq_index]), n, tau_max)
        return self

    def getStripe(self, value: str = "tau"):
        """Image::getStripe (src/Image.cpp:31-41); stripe mode computes tau only."""
        if getattr(self, "_stripe", None) is None:
            raise RuntimeError("run_stripe() first")
        if value != "tau":
            raise ValueError("stripe mode computes tau only")
        return self._stripe

    def getImage(self, value: str, freq_index: int = 0):
        """[n_across][n_along] plane of "tau", "I", "Q", "U", "V" or "l"."""
        if self._images is None:
            raise RuntimeError("run() first")
        return self._images[value][freq_index]

    def getImageSize(self):
        return self.imagePlane.image_size


def make_params(n=100, tau_max=1e4, dt_max=0.0, tau_min=1e-10, output="I", precision="fp64",
                schedule="static", tau_atol=1E-7, tau_rtol=1E-14, atol=1E-9, rtol=1E-9, tau_precision=1.0,
                max_steps=0, block_size=0, refill_threshold=0, ctas_per_sm=0, flags=0) -> A.Params:
    out = {"I": A.OUT_I, "full": A.OUT_FULL}[output] if isinstance(output, str) else int(output)
    prec = {"fp64": A.PREC_FP64, "mixed": A.PREC_MIXED}[precision] if isinstance(precision, str) else int(precision)
    sch = ({"static": A.SCHED_STATIC, "persistent": A.SCHED_PERSISTENT}[schedule]
           if isinstance(schedule, str) else int(schedule))
    return A.Params(n=int(n), output=out, precision=prec, schedule=sch, tau_max=float(tau_max),
                    tau_min=float(tau_min), dt_max=float(dt_max), tau_atol=float(tau_atol),
                    tau_rtol=float(tau_rtol), atol=float(atol), rtol=float(rtol),
                    tau_precision=float(tau_precision), max_steps=int(max_steps),
                    block_size=int(block_size), refill_threshold=int(refill_threshold),
                    ctas_per_sm=int(ctas_per_sm), flags=int(flags))
