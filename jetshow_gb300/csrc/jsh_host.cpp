// jsh_host.cpp -- host half of the library: descriptor validation and
// "model compile" (parameter-only transcendentals evaluated once with the C
// library), image-plane constants, the cosmology integral, defaults and the
// thread-local error message.  Compiled with -ffp-contract=off: the plane
// constants feed the bit-exact geometry kernels.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <cmath>

#include "jsh_model.h"

static thread_local char g_err[512] = "";

void jsh_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

extern "C" const char* jsh_last_error(void) { return g_err; }
extern "C" int jsh_abi_version(void) { return JSH_ABI_VERSION; }

extern "C" void jsh_params_default(jsh_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->n = 100;
  p->output = JSH_OUT_I;
  p->precision = JSH_PREC_FP64;
  p->schedule = JSH_SCHED_STATIC;
  p->tau_max = 1e4;
  p->tau_min = 1e-10;  // pow(10., -10.0) in src/pyjetshow.cpp:148-149
  p->dt_max = 0.0;
  p->tau_atol = 1E-7;
  p->tau_rtol = 1E-14;
  p->atol = 1E-9;
  p->rtol = 1E-9;
  p->tau_precision = 1;
  p->max_steps = 0;
}

namespace {

struct Vd {
  double x, y, z;
};
Vd normalize(Vd a) {
  double n = (a.x * a.x + a.y * a.y) + a.z * a.z;
  if (n > 0.0) {
    double s = sqrt(n);
    return Vd{a.x / s, a.y / s, a.z / s};
  }
  return a;
}

// Modified Bessel I_nu (nu = 0, 1) by the power series (Abramowitz & Stegun 9.6.10).
double bessel_i(int nu, double x) {
  double term = (nu == 0) ? 1.0 : 0.5 * x, sum = term, q = 0.25 * x * x;
  for (int k = 1; k < 500; ++k) {
    term *= q / ((double)k * (double)(k + nu));
    double ns = sum + term;
    if (ns == sum) break;
    sum = ns;
  }
  return sum;
}

bool finite_all(const double* p, int n) {
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(p[i])) return false;
  return true;
}

}  // namespace

int jsh_compile_model(const jsh_model_desc* d, JshModel* m) {
  if (!d || !m) {
    jsh_set_error("null model descriptor");
    return JSH_ERR_INVALID;
  }
  memset(m, 0, sizeof(*m));
  const jsh_geometry_desc& g = d->geometry;
  if (!finite_all(g.origin, 3) || !finite_all(g.direction, 3)) {
    jsh_set_error("geometry origin/direction not finite");
    return JSH_ERR_INVALID;
  }
  m->geo_kind = g.kind;
  m->gox = g.origin[0];
  m->goy = g.origin[1];
  m->goz = g.origin[2];
  // SimulationGeometry has no origin or axis of its own (the hull is
  // revolved about the z axis); its profile is resolved from the context
  Vd dir = g.kind == JSH_GEO_SIMULATION ? Vd{0.0, 0.0, 1.0}
                                        : normalize(Vd{g.direction[0], g.direction[1], g.direction[2]});
  if (!((dir.x * dir.x + dir.y * dir.y) + dir.z * dir.z > 0)) {
    jsh_set_error("geometry direction is zero");
    return JSH_ERR_INVALID;
  }
  m->gdx = dir.x;
  m->gdy = dir.y;
  m->gdz = dir.z;
  m->big_scale = g.big_scale;
  m->r = g.r;
  m->r0 = g.r0;
  m->z0 = g.z0;
  switch (g.kind) {
    case JSH_GEO_CONE:
      m->cone = JshCone{g.origin[0], g.origin[1], g.origin[2], dir.x, dir.y, dir.z, cos(g.angle), g.big_scale};
      break;
    case JSH_GEO_CYLINDER:
      if (!(g.r > 0)) {
        jsh_set_error("cylinder radius must be > 0");
        return JSH_ERR_INVALID;
      }
      break;
    case JSH_GEO_PARABALOID:
      if (!(g.r0 > 0)) {
        jsh_set_error("paraboloid r0 must be > 0");
        return JSH_ERR_INVALID;
      }
      break;
    case JSH_GEO_PARABALOID_CONE: {
      if (!(g.r0 > 0) || !(g.z0 > 0)) {
        jsh_set_error("ParabaloidCone needs r0 > 0 and z0 > 0");
        return JSH_ERR_INVALID;
      }
      // tangent cone at z0 (src/ParabaloidCone.cpp:12-18)
      double r0 = g.r0, z0 = g.z0;
      double shift = -(r0 * sqrt(z0 / JSH_PC) / (0.5 * r0 * pow(z0 * JSH_PC, -0.5)) - z0);
      m->cone = JshCone{g.origin[0] + 0.0, g.origin[1] + 0.0, g.origin[2] + shift, dir.x, dir.y, dir.z,
                        cos(atan(0.5 * r0 * pow(z0 * JSH_PC, -0.5))), g.big_scale};
      break;
    }
    case JSH_GEO_SIMULATION:
      m->hull_id = g.hull_id;
      break;
    default:
      jsh_set_error("unknown geometry kind %d", g.kind);
      return JSH_ERR_INVALID;
  }
  m->b_kind = d->bfield.kind;
  m->n_kind = d->nfield.kind;
  m->v_kind = d->vfield.kind;
  m->b_plasma = d->bfield.in_plasma_frame != 0;
  m->n_plasma = d->nfield.in_plasma_frame != 0;
  for (int i = 0; i < 8; ++i) {
    m->bp[i] = d->bfield.p[i];
    m->np[i] = d->nfield.p[i];
    m->vp[i] = d->vfield.p[i];
  }
  int bk = d->bfield.kind;
  switch (bk) {
    case JSH_B_RANDOM_SCALAR:
    case JSH_B_RANDOM_SCALAR_Z:
    case JSH_B_COMPOSITE_RANDOM_SCALAR_Z:
      m->b_scalar = 1;
      break;
    case JSH_B_CONST_CYLINDER:
    case JSH_B_CONST_CYLINDER_Z:
    case JSH_B_RADIAL_CONICAL:
    case JSH_B_TOROIDAL:
    case JSH_B_HELICAL_CYLINDER:
    case JSH_B_SPIRAL_CONICAL:
    case JSH_B_FORCE_FREE_CYLINDRICAL:
    case JSH_B_HELICAL_CONICAL:
    case JSH_B_SIMULATION:
      m->b_scalar = 0;
      break;
    default:
      jsh_set_error("unknown B-field kind %d", bk);
      return JSH_ERR_INVALID;
  }
  switch (d->nfield.kind) {
    case JSH_N_CONST:
    case JSH_N_BK:
    case JSH_N_BKZ:
    case JSH_N_COMPOSITE_BK:
    case JSH_N_SIMULATION:
      break;
    default:
      jsh_set_error("unknown N-field kind %d", d->nfield.kind);
      return JSH_ERR_INVALID;
  }
  int vk = d->vfield.kind;
  if (!(vk >= JSH_V_CONST_FLAT && vk <= JSH_V_SHEARED_ACC_PARABOLIC_CONST_CONE) && vk != JSH_V_SIMULATION) {
    jsh_set_error("unknown V-field kind %d", vk);
    return JSH_ERR_INVALID;
  }
  double s = d->s;
  if (!std::isfinite(s) || !(s > 0.0)) {
    jsh_set_error("power-law index s must be finite and > 0");
    return JSH_ERR_INVALID;
  }
  m->s = s;
  m->gamma_min = d->gamma_min;
  m->thermal_fraction = d->thermal_fraction;
  // factors exactly as written in src/utils.cpp:40, :47-48, :73, :120, :126-127, :142
  m->fk_i = (pow(3., (s + 1.) / 2.) / 4.) * tgamma(s / 4. + 11. / 6.) * tgamma(s / 4. + 1. / 6.);
  m->rnd_k = sqrt(JSH_PI / 4.) * tgamma((6. + s) / 4.) / tgamma((8. + s) / 4.);
  m->fk_v = pow(3., s / 2.) * (s + 3.) * (s + 2.) / (4. * (s + 1.)) * tgamma(s / 4. + 11. / 12.) *
            tgamma(s / 4. + 7. / 12.);
  m->fe_i = pow(3., s / 2.) / (2. * (s + 1)) * tgamma(s / 4. + 19. / 12.) * tgamma(s / 4. - 1. / 12.);
  m->rnd_e = sqrt(JSH_PI / 4.) * tgamma((5. + s) / 4.) / tgamma((7. + s) / 4.);
  m->fe_v = pow(3., (s - 1.) / 2.) * (s + 2.) / (2. * s) * tgamma(s / 4. + 2. / 3.) * tgamma(s / 4. + 1. / 3.);
  m->kq_ratio = (s + 2.) / (s + 10. / 3);
  m->eq_ratio = (s + 1.0) / (s + 7. / 3.);
  double gm = d->gamma_min;
  m->kfr_factor = (s + 2.) * log(gm) / ((s + 1.) * pow(gm, s + 1.));
  m->kcr_a = (2. / (s - 2.));
  m->kcr_b = pow(gm, 2. - s);
  if (bk == JSH_B_HELICAL_CYLINDER || bk == JSH_B_SPIRAL_CONICAL) m->tan_pitch = tan(d->bfield.p[1]);
  if (bk == JSH_B_FORCE_FREE_CYLINDRICAL) {
    m->bessel0 = bessel_i(0, d->bfield.p[1]);
    m->bessel1 = bessel_i(1, d->bfield.p[1]);
  }
  if (bk == JSH_B_HELICAL_CONICAL) {
    m->sin_pitch = sin(d->bfield.p[2]);
    m->cos_pitch = cos(d->bfield.p[2]);
  }
  if (vk == JSH_V_ACC_PARABOLIC_CONST_CONE || vk == JSH_V_SHEARED_ACC_PARABOLIC_CONST_CONE) {
    double Rz0 = (vk == JSH_V_ACC_PARABOLIC_CONST_CONE) ? d->vfield.p[1] : d->vfield.p[2];
    double z0 = (vk == JSH_V_ACC_PARABOLIC_CONST_CONE) ? d->vfield.p[2] : d->vfield.p[3];
    m->v_cone_oz = (Rz0 * sqrt(z0 / JSH_PC) / (0.5 * Rz0 * pow(z0 * JSH_PC, -0.5)) - z0);
    m->v_theta = atan(sqrt(Rz0 * Rz0 * z0 / JSH_PC) / z0);
  }
  m->grid_b = m->grid_n = m->grid_v = -1;
  if (bk == JSH_B_SIMULATION) {
    m->grid_b = (int32_t)d->bfield.p[0];
    m->fb_p = (int32_t)d->bfield.p[1];
    m->fb_phi = (int32_t)d->bfield.p[2];
  }
  if (d->nfield.kind == JSH_N_SIMULATION) {
    m->grid_n = (int32_t)d->nfield.p[0];
    m->f_n = (int32_t)d->nfield.p[1];
  }
  if (vk == JSH_V_SIMULATION) {
    m->grid_v = (int32_t)d->vfield.p[0];
    m->f_v = (int32_t)d->vfield.p[1];
  }
  // log-domain constants of the mixed-precision coefficients
  {
    const double cb = JSH_Q_E / (2. * JSH_PI * JSH_M_E * JSH_C);  // nu_B per gauss
    const double cp = JSH_Q_E * JSH_Q_E / (JSH_PI * JSH_M_E);     // nu_p^2 per cm^-3
    double fki = m->b_scalar ? m->fk_i * m->rnd_k : m->fk_i;
    double fei = m->b_scalar ? m->fe_i * m->rnd_e : m->fe_i;
    // k_I  = pi cp n cb B (cb B / nu')^(s/2) F / (c nu'^2)
    m->lk_i = log2(JSH_PI * cp * fki / JSH_C) + (1. + s / 2.) * log2(cb);
    // eta_I = pi cp n cb B m_e / c (cb B / nu')^((s-1)/2) F
    m->le_i = log2(JSH_PI * cp * fei * JSH_M_E / JSH_C) + (1. + (s - 1.) / 2.) * log2(cb);
    // eta_V = -pi cp n cb |B| m_e/c cos(theta) (cb B_perp / nu')^(s/2) F_v
    m->le_v = log2(JSH_PI * cp * m->fe_v * JSH_M_E / JSH_C) + (1. + s / 2.) * log2(cb);
    m->lk_cr_b = ((s - 2.) / 2.) * log2(cb);
  }
  // random directions (RandomVectorBField): vector fields only; the wrapper
  // is a plasma-frame field whatever the wrapped one's flag
  // (src/BField.cpp:149-152)
  const jsh_random_desc& rd = d->random;
  m->rnd_kind = rd.kind;
  m->cells_id = -1;
  if (rd.kind != JSH_RND_NONE) {
    if (rd.kind != JSH_RND_CELLS && rd.kind != JSH_RND_POINTS) {
      jsh_set_error("unknown random-field kind %d", rd.kind);
      return JSH_ERR_INVALID;
    }
    if (m->b_scalar) {
      jsh_set_error("random directions wrap a vector B field (RandomVectorBField takes a VectorBField)");
      return JSH_ERR_INVALID;
    }
    if (!std::isfinite(rd.fraction) || !(rd.fraction >= 0.0)) {
      jsh_set_error("random fraction must be finite and >= 0");
      return JSH_ERR_INVALID;
    }
    m->rnd_frac = rd.fraction;
    m->rnd_seed = rd.seed;
    m->b_plasma = 1;
    if (rd.kind == JSH_RND_CELLS) m->cells_id = rd.cells_id;
  }
  m->full_capable = 1;
  return JSH_OK;
}

int jsh_compile_plane(const jsh_plane_desc* d, JshPlane* p) {
  if (!d || !p) {
    jsh_set_error("null plane descriptor");
    return JSH_ERR_INVALID;
  }
  memset(p, 0, sizeof(*p));
  if (d->n_across == 0 || d->n_along == 0) {
    jsh_set_error("image size must be positive");
    return JSH_ERR_INVALID;
  }
  if (d->n_across % 2 != 0) {
    // Image::Image builds n_across/2 positive and n_across/2 negative rows; an
    // odd count indexes past its coordinate table (src/Image.cpp:104-161).
    jsh_set_error("n_across must be even (got %llu)", (unsigned long long)d->n_across);
    return JSH_ERR_INVALID;
  }
  if (d->n_along > (1ull << 24) || d->n_across > (1ull << 24) || d->n_across * d->n_along > (1ull << 34)) {
    jsh_set_error("image too large");
    return JSH_ERR_INVALID;
  }
  if (!std::isfinite(d->lg_pixel_size_start_cm) || !std::isfinite(d->lg_pixel_size_stop_cm) ||
      !std::isfinite(d->los_angle)) {
    jsh_set_error("plane parameters not finite");
    return JSH_ERR_INVALID;
  }
  p->n_across = d->n_across;
  p->n_along = d->n_along;
  p->real_start = pow(10.0, d->lg_pixel_size_start_cm);
  p->real_base = pow(10.0, (d->lg_pixel_size_stop_cm - d->lg_pixel_size_start_cm) / (double)(int)(d->n_along - 1));
  p->inv_sin = 1. / sin(d->los_angle);
  Vd dir = normalize(Vd{-sin(d->los_angle), 0.0, -cos(d->los_angle)});
  Vd dir2 = normalize(dir);
  p->dx = dir.x;
  p->dy = dir.y;
  p->dz = dir.z;
  p->rx = dir2.x;
  p->ry = dir2.y;
  p->rz = dir2.z;
  return JSH_OK;
}

// ------------------------------------------------------------- cosmology
// comoving_transfer_distance2 + mas_to_pc (src/utils.cpp:186-208, :373-378):
// dX/dz = ((Om + (1+z) g_nu)(1+z)^3 + OV)^-1/2 integrated from 0 to z by an
// adaptive Dormand-Prince 5(4) (atol = rtol = 1.49e-8, first step 1e-9).
namespace {
double ctd_rhs(double t, double om, double ov, double gnu) {
  return pow((om + (1. + t) * gnu) * (1. + t) * (1. + t) * (1. + t) + ov, -0.5);
}
}  // namespace

extern "C" double jsh_mas_to_pc(double z, const jsh_cosmology* cosmo) {
  jsh_cosmology dflt = {69.32, 0.2865, 0.7134130719051658, 8.69280948342326e-05};
  if (!cosmo) cosmo = &dflt;
  const double om = cosmo->omega_M, ov = cosmo->omega_V, gnu = cosmo->gamma_nu;
  const double b1 = 35.0 / 384, b3 = 500.0 / 1113, b4 = 125.0 / 192, b5 = -2187.0 / 6784, b6 = 11.0 / 84;
  const double e1 = 71.0 / 57600, e3 = -71.0 / 16695, e4 = 71.0 / 1920, e5 = -17253.0 / 339200, e6 = 22.0 / 525,
               e7 = -1.0 / 40;
  const double tol = 1.49e-8;
  double t = 0.0, x = 0.0, dt = 1E-09;
  double k1 = ctd_rhs(t, om, ov, gnu);
  for (int guard = 0; guard < 1000000 && z - t > 2.220446049250313e-16; ++guard) {
    if ((t + dt) - z > 2.220446049250313e-16) dt = z - t;
    for (int fails = 0; fails < 500; ++fails) {
      // the right-hand side does not depend on x, so only the stage times
      // matter and the a_ij weights drop out
      double k3 = ctd_rhs(t + 0.3 * dt, om, ov, gnu);
      double k4 = ctd_rhs(t + 0.8 * dt, om, ov, gnu);
      double k5 = ctd_rhs(t + 8.0 / 9.0 * dt, om, ov, gnu);
      double k6 = ctd_rhs(t + dt, om, ov, gnu);
      double xn = x + dt * (b1 * k1 + b3 * k3 + b4 * k4 + b5 * k5 + b6 * k6);
      double k7 = k6;
      double err = dt * (e1 * k1 + e3 * k3 + e4 * k4 + e5 * k5 + e6 * k6 + e7 * k7);
      double e = fabs(err) / (tol + tol * (fabs(x) + fabs(dt) * fabs(k1)));
      if (e > 1.0) {
        double f = 0.9 * pow(e, -1.0 / 3.0);
        dt *= (f > 0.2 ? f : 0.2);
        continue;
      }
      x = xn;
      t = t + dt;
      if (e < 0.5) {
        double ee = e > 0.00032 ? e : 0.00032;
        dt *= 9.0 / 10.0 * pow(ee, -1.0 / 5.0);
      }
      k1 = k7;
      break;
    }
  }
  double ctd = (299792.458 / cosmo->H0) * pow(10., 6.) * x;
  return JSH_MAS_TO_RAD * (ctd / (1. + z));
}
