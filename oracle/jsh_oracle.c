/*
 * jsh_oracle.c -- TEST INFRASTRUCTURE (the oracle).  Plain-C FP64
 * restatement of jetshow's per-pixel transfer path.  Only the test suite,
 * the smoke check and bench.py's CPU-baseline leg load it; the product never
 * does.  Compiled with -ffp-contract=off so every expression rounds exactly
 * as written; the evaluation order of each expression is part of the
 * contract the GPU geometry kernels are bit-exact against.
 *
 * Parity is pinned by the reference's Cone::hit golden cases
 * (tests/simple_test.cpp:17-101) and by analytic known answers; for the rest
 * of the transfer path parity unpinned: the reference cannot be built here
 * (Boost.odeint, Eigen, CGAL absent) and holds no golden vectors for it.
 *
 * Third-party arithmetic restated from published sources:
 *  - Dormand & Prince (1980) RK5(4)7M tableau; the continuous extension of
 *    Hairer, Norsett & Wanner, "Solving ODEs I", II.6 (dense output of
 *    DOPRI5, Shampine's coefficients).
 *  - Boost.Odeint (odeint v2; version unpinned by the reference, CI uses
 *    ubuntu:rolling libboost-all-dev) documented semantics: the default error
 *    checker  err = max_i |x_err_i| / (eps_abs + eps_rel (|x_i| + |dt| |dxdt_i|)),
 *    step decrease dt *= max(0.9 err^(-1/(q-1)), 0.2) for err > 1 and increase
 *    dt *= 0.9 max(err, 5^-p)^(-1/p) for err < 0.5 (q = 4 error order,
 *    p = 5 stepper order), 500 consecutive failures abort; integrate_adaptive
 *    truncates the last step to end exactly at t_end; the adaptive range of
 *    a dense-output stepper re-initialises the step to end exactly at t_end.
 */
#include "jsh_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Constants of include/utils.h:17-36 (same values, own names). */
#define JO_MAS_TO_RAD 4.84813681109536e-09
#define JO_PC 3.0856775814671913e+18
#define JO_M_E 9.10938356e-28
#define JO_Q_E 4.80320467299766e-10
#define JO_C 29979245800.0
#define JO_PI 3.141592653589793238462643383279502884

typedef struct { double x, y, z; } v3;

static v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 vmul(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static v3 vdiv(v3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
static double vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static double vsq(v3 a) { return vdot(a, a); }
static double vnorm(v3 a) { return sqrt(vsq(a)); }
static v3 vcross(v3 a, v3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* Eigen's normalize(): divide by sqrt(squaredNorm) when it is positive. */
static v3 vnormalize(v3 a) {
  double n = vsq(a);
  if (n > 0.0) return vdiv(a, sqrt(n));
  return a;
}

/* ====================================================================
 * Image plane: include/logspace.h:25-33, src/Image.cpp:44-194,
 * src/ImagePlane.cpp:11-33, src/Ray.cpp:9-20.
 * ==================================================================== */
typedef struct {
  uint64_t n_across, n_along;
  double* along_size;   /* [n_along]  pyLogspace by repeated multiplication */
  double* along_center; /* [n_along]  partial_sum - size/2                  */
  double* across_pos;   /* [n_across/2][n_along] partial sums - size/2      */
  double inv_sin;       /* 1/sin(los)                                       */
  v3 dir;               /* normalize(-sin los, 0, -cos los)                 */
} plane_t;

static void plane_free(plane_t* p) {
  free(p->along_size);
  free(p->along_center);
  free(p->across_pos);
}

static int plane_build(const jsh_plane_desc* d, plane_t* p) {
  memset(p, 0, sizeof(*p));
  if (d->n_across == 0 || d->n_along == 0 || (d->n_across % 2) != 0) return JSH_ERR_INVALID;
  uint64_t na = d->n_along, nh = d->n_across / 2;
  p->n_across = d->n_across;
  p->n_along = na;
  p->along_size = (double*)malloc(sizeof(double) * na);
  p->along_center = (double*)malloc(sizeof(double) * na);
  p->across_pos = (double*)malloc(sizeof(double) * nh * na);
  if (!p->along_size || !p->along_center || !p->across_pos) { plane_free(p); return JSH_ERR_OOM; }
  /* pyLogspace(start, stop, num, base = 10) */
  double real_start = pow(10.0, d->lg_pixel_size_start_cm);
  double real_base = pow(10.0, (d->lg_pixel_size_stop_cm - d->lg_pixel_size_start_cm) / (double)(int)(na - 1));
  double cur = real_start;
  for (uint64_t j = 0; j < na; ++j) {
    p->along_size[j] = cur;
    cur = cur * real_base;
  }
  /* centres along: std::partial_sum then minus half a size (src/Image.cpp:70-75) */
  double acc = 0.0;
  for (uint64_t j = 0; j < na; ++j) {
    acc = (j == 0) ? p->along_size[0] : acc + p->along_size[j];
    p->along_center[j] = acc - 0.5 * p->along_size[j];
  }
  /* centres across: for column j, partial sums of n_across/2 copies of the
   * column's size (size_along[j] * 1.0) minus half a size (src/Image.cpp:110-126) */
  for (uint64_t j = 0; j < na; ++j) {
    double s = p->along_size[j] * 1.0;
    double a = 0.0;
    for (uint64_t k = 0; k < nh; ++k) {
      a = (k == 0) ? s : a + s;
      p->across_pos[k * na + j] = a - 0.5 * s;
    }
  }
  p->inv_sin = 1. / sin(d->los_angle);
  p->dir = vnormalize(mk(-sin(d->los_angle), 0.0, -cos(d->los_angle)));
  return JSH_OK;
}

/* Ray origin of pixel (row i across, column j along): the pixel coordinate
 * (0, across, along) scaled by (1, 1, 1/sin los) (src/ImagePlane.cpp:16-26).
 * Rows [0, n/2) hold the flipped positive offsets, rows [n/2, n) the
 * negated ones (src/Image.cpp:128-161). */
static v3 plane_origin(const plane_t* p, uint64_t i, uint64_t j) {
  uint64_t nh = p->n_across / 2;
  double across;
  if (i < nh) across = p->across_pos[(nh - i - 1) * p->n_along + j];
  else across = -p->across_pos[(i - nh) * p->n_along + j];
  return mk(1. * 0.0, 1. * across, p->inv_sin * p->along_center[j]);
}

int jo_plane_rays(const jsh_plane_desc* plane, double* origins, double* direction, double* sizes) {
  plane_t p;
  int st = plane_build(plane, &p);
  if (st) return st;
  uint64_t npix = p.n_across * p.n_along;
  for (uint64_t pix = 0; pix < npix; ++pix) {
    uint64_t i = pix / p.n_along, j = pix % p.n_along;
    if (origins) {
      v3 o = plane_origin(&p, i, j);
      origins[3 * pix + 0] = o.x;
      origins[3 * pix + 1] = o.y;
      origins[3 * pix + 2] = o.z;
    }
    if (sizes) sizes[pix] = p.along_size[j];
  }
  if (direction) { direction[0] = p.dir.x; direction[1] = p.dir.y; direction[2] = p.dir.z; }
  plane_free(&p);
  return JSH_OK;
}

/* ====================================================================
 * Geometry: src/Cone.cpp:16-118, src/Geometry.cpp:28-89,
 * src/Cylinder.cpp:9-99, src/Parabaloid.cpp:11-60,
 * src/ParabaloidCone.cpp:12-94, src/Intersection.cpp:26-83.
 * ==================================================================== */
typedef struct { v3 in, out; } seg_t;
typedef struct { int n; seg_t s[2]; uint32_t status; } hits_t;

typedef struct {
  int kind;
  v3 origin, dir;
  double angle, cos_angle, big_scale;
} cone_t;

typedef struct {
  int kind;
  v3 origin, dir;
  double big_scale, r, r0, z0;
  cone_t cone;       /* the cone, or the tangent cone of a ParabaloidCone */
  int hull;          /* SimulationGeometry: registered hull id */
} geo_t;

static void cone_init(cone_t* c, v3 origin, v3 dir, double angle, double scale) {
  c->origin = origin;
  c->dir = vnormalize(dir);
  c->angle = angle;
  c->cos_angle = cos(angle);
  c->big_scale = scale;
}

static v3 ray_point(v3 o, v3 d, double t) { return vadd(o, vmul(d, t)); }

/* Geometry::full_infinite_path / the full-infinite Intersection ctor
 * (src/Geometry.cpp:72-78, src/Intersection.cpp:41-48). */
static seg_t full_infinite(v3 ro, v3 rd, v3 go, double big_scale) {
  v3 diff = vsub(ro, go);
  v3 ref = vsub(diff, vmul(rd, vdot(diff, rd)));
  seg_t s;
  s.in = vsub(ref, vmul(rd, big_scale));
  s.out = vadd(ref, vmul(rd, big_scale));
  return s;
}

static int cone_is_within(const cone_t* c, v3 p) {
  v3 diff = vnormalize(vsub(p, c->origin));
  double cosp = vdot(c->dir, diff);
  return cosp > c->cos_angle || cosp < -c->cos_angle;
}

/* Half-infinite Intersection ctor (src/Intersection.cpp:51-62). */
static seg_t cone_half_infinite(const cone_t* c, v3 rd, v3 point) {
  v3 check = vsub(point, rd);
  seg_t s;
  if (cone_is_within(c, check)) { s.in = vsub(point, vmul(rd, c->big_scale)); s.out = point; }
  else { s.in = point; s.out = vadd(point, vmul(rd, c->big_scale)); }
  return s;
}

/* Cone::hit.  M = d d^T - cos^2(a) I;  c2 = (rd^T M) rd, c1 = (rd^T M) delta,
 * c0 = (delta^T M) delta, each row-vector-times-matrix product summed as
 * (r0 M0j + r1 M1j) + r2 M2j and each dot product as (a0b0 + a1b1) + a2b2. */
static void cone_hit(const cone_t* c, v3 ro, v3 rd, hits_t* h) {
  h->n = 0;
  v3 delta = vsub(ro, c->origin);
  double cos2 = c->cos_angle * c->cos_angle;
  double d[3] = {c->dir.x, c->dir.y, c->dir.z};
  double M[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[i][j] = d[i] * d[j] - cos2 * (i == j ? 1.0 : 0.0);
  double r[3] = {rd.x, rd.y, rd.z}, e[3] = {delta.x, delta.y, delta.z};
  double u[3], w[3];
  for (int j = 0; j < 3; ++j) {
    u[j] = (r[0] * M[0][j] + r[1] * M[1][j]) + r[2] * M[2][j];
    w[j] = (e[0] * M[0][j] + e[1] * M[1][j]) + e[2] * M[2][j];
  }
  double c2 = (u[0] * r[0] + u[1] * r[1]) + u[2] * r[2];
  double c1 = (u[0] * e[0] + u[1] * e[1]) + u[2] * e[2];
  double c0 = (w[0] * e[0] + w[1] * e[1]) + w[2] * e[2];
  double disc = c1 * c1 - c0 * c2;
  if (disc < 0) return;
  if (disc == 0) {
    double t = -c1 / c2;
    v3 point = ray_point(ro, rd, t);
    v3 dp = vsub(point, c->origin);
    /* isMuchSmallerThan(1e-6, 1e-6): squared norm <= (1e-6 * 1e-6)^2 */
    double lim = 1E-06 * 1E-06;
    if (vsq(dp) <= lim * lim && c1 == 0.0) {
      h->n = 1;
      h->s[0] = full_infinite(ro, rd, c->origin, c->big_scale);
    } else {
      h->n = 1;
      h->s[0].in = point;
      h->s[0].out = point;
    }
    return;
  }
  double eps = (c1 > 0 ? 1 : -1);
  double t1 = (-c1 - eps * sqrt(c1 * c1 - c2 * c0)) / (c2);
  double t2 = c0 / (-c1 - eps * sqrt(c1 * c1 - c2 * c0));
  v3 pin = ray_point(ro, rd, fmin(t1, t2));
  v3 pout = ray_point(ro, rd, fmax(t1, t2));
  double cos_ray_cone = vdot(rd, c->dir);
  if (fabs(cos_ray_cone) != 1.) {
    h->n = 1;
    h->s[0].in = pin;
    h->s[0].out = pout;
  } else {
    h->n = 2;
    h->s[0] = cone_half_infinite(c, rd, pout);
    h->s[1] = cone_half_infinite(c, rd, pin);
  }
}

/* Cylinder::hit in pc units; c0 = |w|^2 - r/pc as in src/Cylinder.cpp:53.
 * Unmatched d == 0 cases fall off the end of the reference function (UB);
 * here they are a miss flagged JSH_ST_UB_GEOMETRY. */
static void cylinder_hit(const geo_t* g, v3 ro_cm, v3 rd, hits_t* h) {
  h->n = 0;
  v3 ro = vdiv(ro_cm, JO_PC);
  v3 co = vdiv(g->origin, JO_PC);
  v3 cd = g->dir;
  v3 delta = vsub(ro, co);
  v3 v = vsub(rd, vmul(cd, vdot(rd, cd)));
  double c2 = vsq(v);
  v3 w = vsub(delta, vmul(cd, vdot(delta, cd)));
  double c1 = vdot(v, w);
  double c0 = vsq(w) - g->r / JO_PC;
  double d = c1 * c1 - c0 * c2;
  if (d < 0) return;
  if (d > 0) {
    double eps = (c1 > 0 ? 1 : -1);
    double sq = sqrt(d);
    double t1 = (-c1 - eps * sq) / (c2);
    double t2 = c0 / (-c1 - eps * sq);
    h->n = 1;
    h->s[0].in = ray_point(ro_cm, rd, JO_PC * fmin(t1, t2));
    h->s[0].out = ray_point(ro_cm, rd, JO_PC * fmax(t1, t2));
    return;
  }
  if (c2 == 1 && c1 == 0 && c0 == 0) {
    double t = -c1 / c2;
    v3 p = ray_point(ro_cm, rd, t);
    h->n = 1;
    h->s[0].in = p;
    h->s[0].out = p;
  } else if (c2 == 0 && c1 == 0 && c0 == 0) {
    h->n = 1;
    h->s[0] = full_infinite(ro_cm, rd, g->origin, 100. * g->r);
  } else if (c2 == 0 && c1 == 0 && c0 > 0) {
    return;
  } else if (c2 == 0 && c1 == 0 && c0 <= 0) {
    h->n = 1;
    h->s[0] = full_infinite(ro_cm, rd, g->origin, 100. * g->r);
  } else {
    h->status |= JSH_ST_UB_GEOMETRY;
  }
}

/* intersection() of src/Geometry.cpp:28-69: general quadric
 * A x^2 + B y^2 + C z^2 + D xy + E xz + F yz + G x + H y + I z + J = 0 with
 * the textbook quadratic formula; returns the number of roots in ts. */
static int quadric_roots(v3 R0, v3 Rd, double A, double B, double C, double D, double E,
                         double F, double G, double H, double I, double J, double ts[2]) {
  double x0 = R0.x, y0 = R0.y, z0 = R0.z;
  double xd = Rd.x, yd = Rd.y, zd = Rd.z;
  double Aq = A * xd * xd + B * yd * yd + C * zd * zd + D * xd * yd + E * xd * zd + F * yd * zd;
  double Bq = 2 * A * x0 * xd + 2 * B * y0 * yd + 2 * C * z0 * zd + D * (x0 * yd + y0 * xd) +
              E * x0 * zd + F * (y0 * zd + yd * z0) + G * xd + H * yd + I * zd;
  double Cq = A * x0 * x0 + B * y0 * y0 + C * z0 * z0 + D * x0 * y0 + E * x0 * z0 + F * y0 * z0 +
              G * x0 + H * y0 + I * z0 + J;
  double Dscr = Bq * Bq - 4 * Aq * Cq;
  if (Aq == 0) { ts[0] = -Cq / Bq; return 1; }
  if (Dscr < 0) return 0;
  double t0 = (-Bq - sqrt(Dscr)) / (2 * Aq);
  if (t0 > 0) { ts[0] = t0; return 1; }
  ts[0] = t0;
  ts[1] = (-Bq + sqrt(Dscr)) / (2 * Aq);
  return 2;
}

/* Parabaloid::hit: x^2 + y^2 - (r0^2/pc) z = 0; a single root is a miss. */
static void parabaloid_hit(double r0, v3 ro, v3 rd, hits_t* h) {
  h->n = 0;
  double ts[2];
  int n = quadric_roots(ro, rd, 1., 1., 0., 0., 0., 0., 0., 0., -r0 * r0 / JO_PC, 0.0, ts);
  if (n == 2) {
    h->n = 1;
    h->s[0].in = ray_point(ro, rd, fmin(ts[0], ts[1]));
    h->s[0].out = ray_point(ro, rd, fmax(ts[0], ts[1]));
  }
}

/* ParabaloidCone::hit (src/ParabaloidCone.cpp:45-94).  The reference
 * dereferences an empty cone list when only the paraboloid is hit (UB);
 * here that is a miss flagged JSH_ST_UB_GEOMETRY. */
static void parabaloid_cone_hit(const geo_t* g, v3 ro, v3 rd, hits_t* h) {
  hits_t hc = {0}, hp = {0};
  cone_hit(&g->cone, ro, rd, &hc);
  parabaloid_hit(g->r0, ro, rd, &hp);
  h->n = 0;
  h->status |= hc.status | hp.status;
  if (hc.n == 0 && hp.n == 0) return;
  if (hc.n != 0 && hp.n == 0) {
    if (hc.s[0].in.z > g->z0) *h = hc;
    return;
  }
  if (hc.n == 0) { h->status |= JSH_ST_UB_GEOMETRY; return; }
  v3 pin, pout;
  pin = (hp.s[0].in.z > g->z0) ? hc.s[0].in : hp.s[0].in;
  pout = (hp.s[0].out.z < g->z0) ? hp.s[0].out : hc.s[0].out;
  h->n = 1;
  h->s[0].in = pin;
  h->s[0].out = pout;
}

/* --------------------------------------------------------------------
 * SimulationGeometry (src/Geometry.cpp:92-132; hull built at
 * src/main.cpp:880-897): the convex hull of the (z, r) points revolved at
 * n_circle azimuths phi_j = 2 pi j / n_circle, (r sin phi_j, r cos phi_j, z),
 * intersected with the ray's line in pc.  The hull of such a cloud is
 * {(x, y, z): max_k g_k . (x, y) <= R(z), z_min <= z <= z_max}, g_k the
 * face normals of the regular n_circle-gon at (2k + 1) pi / n_circle over
 * cos(pi / n_circle) and R the upper envelope of the 2-D hull of the (z, r)
 * points: both support functions are max_i (r_i |u_xy| c(psi) + z_i u_z),
 * c(psi) = max_j cos(phi_j - psi).  tests/test_hull.py checks the form
 * against scipy's Qhull hull of the revolved cloud itself.
 * -------------------------------------------------------------------- */
#define JO_MAX_HULLS 16
typedef struct {
  int used, m, n_circle;
  double *vz, *vR, *abc, *g;
  double z_min, z_max;
} jo_hull;
static jo_hull g_hulls[JO_MAX_HULLS];

static int cmp_zr(const void* pa, const void* pb) {
  const double* a = (const double*)pa;
  const double* b = (const double*)pb;
  if (a[0] != b[0]) return a[0] < b[0] ? -1 : 1;
  if (a[1] != b[1]) return a[1] < b[1] ? -1 : 1;
  return 0;
}

int jo_hull_register(int32_t hull_id, const double* zr, int64_t n, int32_t n_circle) {
  if (hull_id < 0 || hull_id >= JO_MAX_HULLS || n < 2 || n_circle < 3 || n_circle > 4096) return JSH_ERR_INVALID;
  for (int64_t i = 0; i < n; ++i)
    if (!isfinite(zr[2 * i]) || !isfinite(zr[2 * i + 1]) || zr[2 * i + 1] < 0) return JSH_ERR_INVALID;
  double* p = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  memcpy(p, zr, sizeof(double) * 2 * (size_t)n);
  qsort(p, (size_t)n, 2 * sizeof(double), cmp_zr);
  /* per z only its largest r can lie on the upper envelope */
  int64_t nq = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (i + 1 < n && p[2 * (i + 1)] == p[2 * i]) continue;
    p[2 * nq] = p[2 * i];
    p[2 * nq + 1] = p[2 * i + 1];
    nq++;
  }
  if (nq < 2) { free(p); return JSH_ERR_INVALID; }
  /* Andrew's monotone chain, upper hull of (z, r); collinear points dropped */
  double* h = (double*)malloc(sizeof(double) * 2 * (size_t)nq);
  int64_t nh = 0;
  for (int64_t i = 0; i < nq; ++i) {
    double cz = p[2 * i], cr = p[2 * i + 1];
    while (nh >= 2) {
      double oz = h[2 * (nh - 2)], orr = h[2 * (nh - 2) + 1], az = h[2 * (nh - 1)], ar = h[2 * (nh - 1) + 1];
      double cross = (az - oz) * (cr - orr) - (ar - orr) * (cz - oz);
      if (cross >= 0) nh--;
      else break;
    }
    h[2 * nh] = cz;
    h[2 * nh + 1] = cr;
    nh++;
  }
  free(p);
  jo_hull* H = &g_hulls[hull_id];
  if (H->used) { free(H->vz); free(H->vR); free(H->abc); free(H->g); }
  int m = (int)(nh - 1);
  H->m = m;
  H->n_circle = n_circle;
  H->vz = (double*)malloc(sizeof(double) * (size_t)(m + 1));
  H->vR = (double*)malloc(sizeof(double) * (size_t)(m + 1));
  H->abc = (double*)malloc(sizeof(double) * 3 * (size_t)m);
  H->g = (double*)malloc(sizeof(double) * 2 * (size_t)n_circle);
  for (int i = 0; i <= m; ++i) { H->vz[i] = h[2 * i]; H->vR[i] = h[2 * i + 1]; }
  free(h);
  for (int e = 0; e < m; ++e) {
    double a = H->vz[e + 1] - H->vz[e];
    double b = -(H->vR[e + 1] - H->vR[e]);
    H->abc[3 * e] = a;
    H->abc[3 * e + 1] = b;
    H->abc[3 * e + 2] = a * H->vR[e] + b * H->vz[e];
  }
  double inv_cos = 1.0 / cos(JO_PI / (double)n_circle);
  for (int k = 0; k < n_circle; ++k) {
    double ang = ((2.0 * k + 1.0) * JO_PI) / (double)n_circle;
    H->g[2 * k] = sin(ang) * inv_cos;
    H->g[2 * k + 1] = cos(ang) * inv_cos;
  }
  H->z_min = H->vz[0];
  H->z_max = H->vz[m];
  H->used = 1;
  return JSH_OK;
}

int jo_hull_profile(int32_t hull_id, double* vz, double* vR, int32_t* m) {
  if (hull_id < 0 || hull_id >= JO_MAX_HULLS || !g_hulls[hull_id].used) return JSH_ERR_NOT_FOUND;
  const jo_hull* H = &g_hulls[hull_id];
  if (m) *m = H->m;
  for (int i = 0; i <= H->m; ++i) {
    if (vz) vz[i] = H->vz[i];
    if (vR) vR[i] = H->vR[i];
  }
  return JSH_OK;
}

/* D(z_i) = R_i - (A + B z_i): R minus the line's sector coordinate */
static double hull_D(const jo_hull* H, int i, double A, double B) { return H->vR[i] - (A + B * H->vz[i]); }

static double hull_edge_t(const jo_hull* H, int e, double u0, double u1, double oz, double dz) {
  double a = H->abc[3 * e], b = H->abc[3 * e + 1], c = H->abc[3 * e + 2];
  double alpha = (a * u0 + b * oz) - c;
  double beta = a * u1 + b * dz;
  if (beta == 0.0) return (H->vz[e] - oz) / dz;
  return -alpha / beta;
}

/* Per sector k the line's slab interval: along z (d_z != 0) D is concave
 * and piecewise linear with breaks at the profile vertices; its maximum
 * vertex and the sign changes on both sides (binary searches) give the
 * crossed edges (or the caps z_min, z_max).  The segment is
 * [max_k t_in, min_k t_out]; point_in is the point of smaller t. */
static void simulation_hit(const jo_hull* H, v3 ro_cm, v3 rd, hits_t* h) {
  v3 o = vdiv(ro_cm, JO_PC);
  int m = H->m;
  double tlo = -INFINITY, thi = INFINITY;
  if (rd.z == 0.0) {
    if (!(o.z >= H->z_min && o.z <= H->z_max)) return;
    int lo = 0, hi = m;
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (H->vz[mid] <= o.z) lo = mid;
      else hi = mid;
    }
    double a = H->abc[3 * lo], b = H->abc[3 * lo + 1], c = H->abc[3 * lo + 2];
    double R0 = (c - b * o.z) / a;
    for (int k = 0; k < H->n_circle; ++k) {
      double gx = H->g[2 * k], gy = H->g[2 * k + 1];
      double u0 = gx * o.x + gy * o.y, u1 = gx * rd.x + gy * rd.y;
      if (u1 > 0.0) thi = fmin(thi, (R0 - u0) / u1);
      else if (u1 < 0.0) tlo = fmax(tlo, (R0 - u0) / u1);
      else if (u0 > R0) return;
    }
  } else {
    double t_zmin = (H->z_min - o.z) / rd.z, t_zmax = (H->z_max - o.z) / rd.z;
    for (int k = 0; k < H->n_circle; ++k) {
      double gx = H->g[2 * k], gy = H->g[2 * k + 1];
      double u0 = gx * o.x + gy * o.y, u1 = gx * rd.x + gy * rd.y;
      double B = u1 / rd.z, A = u0 - B * o.z;
      int lo = 0, hi = m;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if ((H->vR[mid + 1] - H->vR[mid]) - B * (H->vz[mid + 1] - H->vz[mid]) < 0.0) hi = mid;
        else lo = mid + 1;
      }
      int top = lo;
      if (!(hull_D(H, top, A, B) >= 0.0)) return;
      double ta, tb;
      if (hull_D(H, 0, A, B) >= 0.0) {
        ta = t_zmin;
      } else {
        int l = 0, r = top;
        while (r - l > 1) {
          int mid = (l + r) >> 1;
          if (hull_D(H, mid, A, B) >= 0.0) r = mid;
          else l = mid;
        }
        ta = hull_edge_t(H, l, u0, u1, o.z, rd.z);
      }
      if (hull_D(H, m, A, B) >= 0.0) {
        tb = t_zmax;
      } else {
        int l = top, r = m;
        while (r - l > 1) {
          int mid = (l + r) >> 1;
          if (hull_D(H, mid, A, B) >= 0.0) l = mid;
          else r = mid;
        }
        tb = hull_edge_t(H, l, u0, u1, o.z, rd.z);
      }
      tlo = fmax(tlo, fmin(ta, tb));
      thi = fmin(thi, fmax(ta, tb));
    }
  }
  if (!(tlo < thi)) {
    if (tlo == thi) h->status |= JSH_ST_UB_GEOMETRY;
    return;
  }
  h->n = 1;
  h->s[0].in = vmul(ray_point(o, rd, tlo), JO_PC);
  h->s[0].out = vmul(ray_point(o, rd, thi), JO_PC);
}

static int geo_init(const jsh_geometry_desc* d, geo_t* g) {
  memset(g, 0, sizeof(*g));
  g->kind = d->kind;
  g->origin = mk(d->origin[0], d->origin[1], d->origin[2]);
  g->dir = vnormalize(mk(d->direction[0], d->direction[1], d->direction[2]));
  g->big_scale = d->big_scale;
  g->r = d->r;
  g->r0 = d->r0;
  g->z0 = d->z0;
  switch (d->kind) {
    case JSH_GEO_CONE:
      cone_init(&g->cone, g->origin, mk(d->direction[0], d->direction[1], d->direction[2]), d->angle,
                d->big_scale);
      return JSH_OK;
    case JSH_GEO_CYLINDER:
    case JSH_GEO_PARABALOID:
      return JSH_OK;
    case JSH_GEO_SIMULATION:
      if (d->hull_id < 0 || d->hull_id >= JO_MAX_HULLS || !g_hulls[d->hull_id].used) return JSH_ERR_NOT_FOUND;
      g->hull = d->hull_id;
      return JSH_OK;
    case JSH_GEO_PARABALOID_CONE: {
      /* tangent cone at z0 (src/ParabaloidCone.cpp:12-18) */
      double r0 = d->r0, z0 = d->z0;
      double shift = -(r0 * sqrt(z0 / JO_PC) / (0.5 * r0 * pow(z0 * JO_PC, -0.5)) - z0);
      v3 co = vadd(g->origin, mk(0, 0, shift));
      cone_init(&g->cone, co, mk(d->direction[0], d->direction[1], d->direction[2]),
                atan(0.5 * r0 * pow(z0 * JO_PC, -0.5)), d->big_scale);
      return JSH_OK;
    }
    default:
      return JSH_ERR_INVALID;
  }
}

static void geo_hit(const geo_t* g, v3 ro, v3 rd, hits_t* h) {
  h->n = 0;
  h->status = 0;
  switch (g->kind) {
    case JSH_GEO_CONE: cone_hit(&g->cone, ro, rd, h); break;
    case JSH_GEO_CYLINDER: cylinder_hit(g, ro, rd, h); break;
    case JSH_GEO_PARABALOID: parabaloid_hit(g->r0, ro, rd, h); break;
    case JSH_GEO_PARABALOID_CONE: parabaloid_cone_hit(g, ro, rd, h); break;
    case JSH_GEO_SIMULATION: simulation_hit(&g_hulls[g->hull], ro, rd, h); break;
    default: break;
  }
}

int jo_hit_rays(const jsh_model_desc* model, const double* origins, const double* directions,
                int64_t n, int32_t* n_seg, double* seg, uint32_t* status) {
  geo_t g;
  int st = geo_init(&model->geometry, &g);
  if (st) return st;
  for (int64_t i = 0; i < n; ++i) {
    v3 ro = mk(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]);
    v3 rd = vnormalize(mk(directions[3 * i], directions[3 * i + 1], directions[3 * i + 2]));
    hits_t h;
    geo_hit(&g, ro, rd, &h);
    if (n_seg) n_seg[i] = h.n;
    if (status) status[i] = h.status | (h.n ? JSH_ST_HIT : 0u);
    if (seg) {
      for (int k = 0; k < 2; ++k) {
        double* s = seg + 12 * i + 6 * k;
        if (k < h.n) {
          s[0] = h.s[k].in.x; s[1] = h.s[k].in.y; s[2] = h.s[k].in.z;
          s[3] = h.s[k].out.x; s[4] = h.s[k].out.y; s[5] = h.s[k].out.z;
        } else {
          for (int q = 0; q < 6; ++q) s[q] = 0.0;
        }
      }
    }
  }
  return JSH_OK;
}

/* ====================================================================
 * Gridded fields (SimulationInterpolater, src/SimulationInterpolater.cpp:43-102):
 * (x, y, z) -> (z/pc, hypot(x, y)/pc); the containing triangle of a
 * Delaunay triangulation; barycentric weights; nan_value outside the hull
 * or on NaN.  Point location here is a plain uniform bucket grid.
 * ==================================================================== */
#define JO_MAX_GRIDS 16
typedef struct {
  int used;
  int64_t n, n_tri;
  int32_t n_fields;
  double* xy;
  float* val;
  int32_t* tri;
  double x0, y0, hx, hy;
  int32_t nbx, nby;
  int64_t* bstart; /* [nbx*nby+1] */
  int32_t* bitems;
} jo_grid;

static jo_grid g_grids[JO_MAX_GRIDS];

static void grid_free(jo_grid* G) {
  free(G->xy); free(G->val); free(G->tri); free(G->bstart); free(G->bitems);
  memset(G, 0, sizeof(*G));
}

int jo_grid_register(int32_t grid_id, const double* xy, int64_t n, const float* values,
                     int32_t n_fields, const int32_t* tri, int64_t n_tri) {
  if (grid_id < 0 || grid_id >= JO_MAX_GRIDS || n < 3 || n_tri < 1 || n_fields < 1)
    return JSH_ERR_INVALID;
  jo_grid* G = &g_grids[grid_id];
  if (G->used) grid_free(G);
  G->n = n; G->n_tri = n_tri; G->n_fields = n_fields;
  G->xy = (double*)malloc(sizeof(double) * 2 * n);
  G->val = (float*)malloc(sizeof(float) * n * n_fields);
  G->tri = (int32_t*)malloc(sizeof(int32_t) * 3 * n_tri);
  memcpy(G->xy, xy, sizeof(double) * 2 * n);
  memcpy(G->val, values, sizeof(float) * n * n_fields);
  memcpy(G->tri, tri, sizeof(int32_t) * 3 * n_tri);
  double xmin = xy[0], xmax = xy[0], ymin = xy[1], ymax = xy[1];
  for (int64_t i = 1; i < n; ++i) {
    xmin = fmin(xmin, xy[2 * i]); xmax = fmax(xmax, xy[2 * i]);
    ymin = fmin(ymin, xy[2 * i + 1]); ymax = fmax(ymax, xy[2 * i + 1]);
  }
  int32_t nb = (int32_t)ceil(sqrt((double)n_tri / 2.0));
  if (nb < 1) nb = 1;
  G->nbx = nb; G->nby = nb;
  G->x0 = xmin; G->y0 = ymin;
  G->hx = (xmax - xmin) / nb; G->hy = (ymax - ymin) / nb;
  if (G->hx <= 0) G->hx = 1;
  if (G->hy <= 0) G->hy = 1;
  int64_t nbk = (int64_t)nb * nb;
  int64_t* cnt = (int64_t*)calloc(nbk + 1, sizeof(int64_t));
  for (int pass = 0; pass < 2; ++pass) {
    for (int64_t t = 0; t < n_tri; ++t) {
      double bx0 = 1e300, bx1 = -1e300, by0 = 1e300, by1 = -1e300;
      for (int k = 0; k < 3; ++k) {
        int32_t v = tri[3 * t + k];
        bx0 = fmin(bx0, xy[2 * v]); bx1 = fmax(bx1, xy[2 * v]);
        by0 = fmin(by0, xy[2 * v + 1]); by1 = fmax(by1, xy[2 * v + 1]);
      }
      int32_t i0 = (int32_t)floor((bx0 - G->x0) / G->hx) - 1, i1 = (int32_t)floor((bx1 - G->x0) / G->hx) + 1;
      int32_t j0 = (int32_t)floor((by0 - G->y0) / G->hy) - 1, j1 = (int32_t)floor((by1 - G->y0) / G->hy) + 1;
      if (i0 < 0) i0 = 0;
      if (j0 < 0) j0 = 0;
      if (i1 >= nb) i1 = nb - 1;
      if (j1 >= nb) j1 = nb - 1;
      for (int32_t j = j0; j <= j1; ++j)
        for (int32_t i = i0; i <= i1; ++i) {
          int64_t b = (int64_t)j * nb + i;
          if (pass == 0) cnt[b + 1]++;
          else G->bitems[cnt[b]++] = (int32_t)t;
        }
    }
    if (pass == 0) {
      for (int64_t b = 0; b < nbk; ++b) cnt[b + 1] += cnt[b];
      G->bstart = (int64_t*)malloc(sizeof(int64_t) * (nbk + 1));
      memcpy(G->bstart, cnt, sizeof(int64_t) * (nbk + 1));
      G->bitems = (int32_t*)malloc(sizeof(int32_t) * (cnt[nbk] ? cnt[nbk] : 1));
    }
  }
  free(cnt);
  G->used = 1;
  return JSH_OK;
}

static double orient2(double ax, double ay, double bx, double by, double cx, double cy) {
  return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
}

double jo_grid_value(int32_t grid_id, int32_t field, double px, double py, double nan_value) {
  if (grid_id < 0 || grid_id >= JO_MAX_GRIDS || !g_grids[grid_id].used) return nan_value;
  const jo_grid* G = &g_grids[grid_id];
  if (field < 0 || field >= G->n_fields) return nan_value;
  int32_t i = (int32_t)floor((px - G->x0) / G->hx), j = (int32_t)floor((py - G->y0) / G->hy);
  if (!(px >= G->x0 && py >= G->y0)) return nan_value;
  if (i >= G->nbx) i = G->nbx - 1;
  if (j >= G->nby) j = G->nby - 1;
  if (i < 0 || j < 0) return nan_value;
  int64_t b = (int64_t)j * G->nbx + i;
  for (int64_t q = G->bstart[b]; q < G->bstart[b + 1]; ++q) {
    int32_t t = G->bitems[q];
    int32_t v0 = G->tri[3 * t], v1 = G->tri[3 * t + 1], v2 = G->tri[3 * t + 2];
    double ax = G->xy[2 * v0], ay = G->xy[2 * v0 + 1];
    double bx = G->xy[2 * v1], by = G->xy[2 * v1 + 1];
    double cx = G->xy[2 * v2], cy = G->xy[2 * v2 + 1];
    double area = orient2(ax, ay, bx, by, cx, cy);
    if (area == 0) continue;
    double w0 = orient2(px, py, bx, by, cx, cy) / area;
    double w1 = orient2(ax, ay, px, py, cx, cy) / area;
    double w2 = orient2(ax, ay, bx, by, px, py) / area;
    if (w0 < 0 || w1 < 0 || w2 < 0) continue;
    double val = w0 * (double)G->val[(int64_t)v0 * G->n_fields + field] +
                 w1 * (double)G->val[(int64_t)v1 * G->n_fields + field] +
                 w2 * (double)G->val[(int64_t)v2 * G->n_fields + field];
    if (isnan(val)) return nan_value;
    return val;
  }
  return nan_value;
}

/* hypot(x, y) of src/SimulationInterpolater.cpp:49 as sqrt(x*x + y*y), each
 * operation rounded once (-ffp-contract=off): within an ulp of a libm hypot
 * at these magnitudes (the reference's libm is unpinned), and the order the
 * device rounds in, so device and oracle locate the same triangle. */
static double sim_value(int32_t grid, int32_t field, v3 p, double nan_value) {
  double x = p.x / JO_PC, y = p.y / JO_PC, z = p.z / JO_PC;
  double r = sqrt(x * x + y * y);
  return jo_grid_value(grid, field, z, r, nan_value);
}

/* ====================================================================
 * Random directions of RandomVectorBField (src/BField.cpp:149-193) and the
 * cells of RandomCellsInSphere (src/Cells.cpp:5-47, src/utils.cpp:249-312).
 * The reference draws from Boost Mersenne Twisters (per OpenMP thread for
 * PointsRandomVectorBField); the GB300 build replaces them with the
 * counter-based Philox4x32-10 generator (Salmon et al., SC'11), restated
 * here from the published algorithm: ten rounds of
 *   (c0, c1, c2, c3) -> (hi(M1 c2) ^ c1 ^ k0, lo(M1 c2), hi(M0 c0) ^ c3 ^ k1, lo(M0 c0)),
 * M0 = 0xD2511F53, M1 = 0xCD9E8D57, the key (k0, k1) advanced by
 * (0x9E3779B9, 0xBB67AE85) between rounds.  Uniforms U = (x + 1/2) 2^-32;
 * directions by rejection from the cube [-1, 1]^3 into the unit ball, then
 * divided by the norm (every operation rounded once, -ffp-contract=off).
 * Counters: a cell's direction (cell, 0xFFFFFFFF, 0, 1 << 24 | attempt), a
 * cell's position uniforms (cell, 0xFFFFFFFE, 0, 2 << 24), the direction of
 * one right-hand-side evaluation (pixel, frequency, evaluation index,
 * 1 << 24 | attempt); the key is the seed.
 * ==================================================================== */
typedef struct { uint32_t c[4]; } jo_u4;

static jo_u4 jo_philox(jo_u4 x, uint64_t seed) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t)0xD2511F53u * x.c[0], p1 = (uint64_t)0xCD9E8D57u * x.c[2];
    jo_u4 y;
    y.c[0] = (uint32_t)(p1 >> 32) ^ x.c[1] ^ k0;
    y.c[1] = (uint32_t)p1;
    y.c[2] = (uint32_t)(p0 >> 32) ^ x.c[3] ^ k1;
    y.c[3] = (uint32_t)p0;
    x = y;
  }
  return x;
}

int jo_philox4x32(const uint32_t* ctr, uint64_t key, uint32_t* out) {
  jo_u4 x = {{ctr[0], ctr[1], ctr[2], ctr[3]}};
  jo_u4 y = jo_philox(x, key);
  for (int i = 0; i < 4; ++i) out[i] = y.c[i];
  return JSH_OK;
}

static double jo_u01(uint32_t x) { return ((double)x + 0.5) * 2.3283064365386962890625e-10; }

void jo_random_direction(uint64_t seed, uint32_t k0, uint32_t k1, uint32_t k2, double* n) {
  for (uint32_t a = 0; a < 64u; ++a) {
    jo_u4 x = {{k0, k1, k2, 0x01000000u | a}};
    jo_u4 r = jo_philox(x, seed);
    double cx = 2.0 * jo_u01(r.c[0]) - 1.0, cy = 2.0 * jo_u01(r.c[1]) - 1.0, cz = 2.0 * jo_u01(r.c[2]) - 1.0;
    double r2 = (cx * cx + cy * cy) + cz * cz;
    if (r2 > 0.0 && r2 <= 1.0) {
      double s = sqrt(r2);
      n[0] = cx / s; n[1] = cy / s; n[2] = cz / s;
      return;
    }
  }
  n[0] = 0.0; n[1] = 0.0; n[2] = 1.0;
}

int jo_cells_generate(int64_t n, double r_min, double r_max, double theta_max, double exponent, uint64_t seed,
                      double* points, double* dirs) {
  if (n < 1 || !points || !dirs || exponent == 3.0) return JSH_ERR_INVALID;
  /* generate_random_points_sphere (src/utils.cpp:267-312) */
  double c = theta_max > 0 ? cos(theta_max) : 1.0;
  for (int64_t j = 0; j < n; ++j) {
    jo_u4 x = {{(uint32_t)j, 0xFFFFFFFEu, 0u, 0x02000000u}};
    jo_u4 u = jo_philox(x, seed);
    double r = r_min + (r_max - r_min) * jo_u01(u.c[0]);
    double phi = 2.0 * JO_PI * jo_u01(u.c[1]);
    double uu = (1.0 - c) * (2.0 * jo_u01(u.c[2]) - 1.0);
    if (uu < 0.0) uu = uu - c;
    else uu = uu + c;
    double theta = acos(uu);
    r = pow(r, 1. / (3.0 - exponent));
    points[3 * j] = r * sin(theta) * cos(phi);
    points[3 * j + 1] = r * sin(theta) * sin(phi);
    points[3 * j + 2] = r * cos(theta);
    /* generate_random_directions (src/utils.cpp:249-261) */
    jo_random_direction(seed, (uint32_t)j, 0xFFFFFFFFu, 0u, dirs + 3 * j);
  }
  return JSH_OK;
}

#define JO_MAX_CELLS 16
typedef struct { int used; int64_t n; double* p; double* dir; } jo_cells;
static jo_cells g_cells[JO_MAX_CELLS];

int jo_cells_register(int32_t id, const double* points, const double* dirs, int64_t n) {
  if (id < 0 || id >= JO_MAX_CELLS || n < 1) return JSH_ERR_INVALID;
  jo_cells* C = &g_cells[id];
  if (C->used) { free(C->p); free(C->dir); }
  C->p = (double*)malloc(sizeof(double) * 3 * n);
  C->dir = (double*)malloc(sizeof(double) * 3 * n);
  memcpy(C->p, points, sizeof(double) * 3 * n);
  memcpy(C->dir, dirs, sizeof(double) * 3 * n);
  C->n = n;
  C->used = 1;
  return JSH_OK;
}

/* RandomCells::getID (src/Cells.cpp:13-18): the smallest squared distance
 * over every cell, the lowest index among equals. */
int64_t jo_cells_nearest(int32_t id, const double* q) {
  if (id < 0 || id >= JO_MAX_CELLS || !g_cells[id].used) return -1;
  const jo_cells* C = &g_cells[id];
  double best = INFINITY;
  int64_t bi = 0;
  for (int64_t i = 0; i < C->n; ++i) {
    double dx = q[0] - C->p[3 * i], dy = q[1] - C->p[3 * i + 1], dz = q[2] - C->p[3 * i + 2];
    double d2 = (dx * dx + dy * dy) + dz * dz;
    if (d2 < best) { best = d2; bi = i; }
  }
  return bi;
}

/* ====================================================================
 * Fields: src/VField.cpp:25-274, src/BField.cpp:35-224, src/NField.cpp:5-60.
 * ==================================================================== */
typedef struct {
  jsh_model_desc d;
  geo_t geo;
  int b_scalar;
  double fk_i, fk_v, fe_i, fe_v;   /* tgamma factors of k_i, k_v, eta_i, eta_v */
  double rnd_k, rnd_e;             /* angle-average factors of scalar-B k_i, eta_i */
  double kq_ratio, eq_ratio;       /* (s+2)/(s+10/3), (s+1)/(s+7/3) */
  double kfr_factor;               /* (s+2) ln(g)/((s+1) g^(s+1)) */
  double kcr_a, kcr_b;             /* 2/(s-2), g^(2-s) */
  double tan_pitch, bessel0, bessel1, sin_pitch, cos_pitch;
  double v_cone_oz, v_theta;       /* composite velocity fields */
} model_t;

/* Modified Bessel functions I0, I1 by their power series (Abramowitz &
 * Stegun 9.6.10), summed until the terms stop changing the sum. */
static double bessel_i(int nu, double x) {
  double term = (nu == 0) ? 1.0 : 0.5 * x, sum = term, q = 0.25 * x * x;
  for (int k = 1; k < 500; ++k) {
    term *= q / ((double)k * (double)(k + nu));
    double ns = sum + term;
    if (ns == sum) break;
    sum = ns;
  }
  return sum;
}

static int model_init(const jsh_model_desc* d, model_t* m) {
  memset(m, 0, sizeof(*m));
  m->d = *d;
  int st = geo_init(&d->geometry, &m->geo);
  if (st) return st;
  double s = d->s;
  int bk = d->bfield.kind;
  m->b_scalar = (bk == JSH_B_RANDOM_SCALAR || bk == JSH_B_RANDOM_SCALAR_Z || bk == JSH_B_COMPOSITE_RANDOM_SCALAR_Z);
  /* factors exactly as written in src/utils.cpp:40, :47-48, :73, :120, :126-127, :142 */
  m->fk_i = (pow(3., (s + 1.) / 2.) / 4.) * tgamma(s / 4. + 11. / 6.) * tgamma(s / 4. + 1. / 6.);
  m->rnd_k = sqrt(JO_PI / 4.) * tgamma((6. + s) / 4.) / tgamma((8. + s) / 4.);
  m->fk_v = pow(3., s / 2.) * (s + 3.) * (s + 2.) / (4. * (s + 1.)) * tgamma(s / 4. + 11. / 12.) * tgamma(s / 4. + 7. / 12.);
  m->fe_i = pow(3., s / 2.) / (2. * (s + 1)) * tgamma(s / 4. + 19. / 12.) * tgamma(s / 4. - 1. / 12.);
  m->rnd_e = sqrt(JO_PI / 4.) * tgamma((5. + s) / 4.) / tgamma((7. + s) / 4.);
  m->fe_v = pow(3., (s - 1.) / 2.) * (s + 2.) / (2. * s) * tgamma(s / 4. + 2. / 3.) * tgamma(s / 4. + 1. / 3.);
  m->kq_ratio = (s + 2.) / (s + 10. / 3);
  m->eq_ratio = (s + 1.0) / (s + 7. / 3.);
  double g = d->gamma_min;
  m->kfr_factor = (s + 2.) * log(g) / ((s + 1.) * pow(g, s + 1.));
  m->kcr_a = (2. / (s - 2.));
  m->kcr_b = pow(g, 2. - s);
  if (bk == JSH_B_HELICAL_CYLINDER || bk == JSH_B_SPIRAL_CONICAL) m->tan_pitch = tan(d->bfield.p[1]);
  if (bk == JSH_B_FORCE_FREE_CYLINDRICAL) {
    m->bessel0 = bessel_i(0, d->bfield.p[1]);
    m->bessel1 = bessel_i(1, d->bfield.p[1]);
  }
  if (bk == JSH_B_HELICAL_CONICAL) { m->sin_pitch = sin(d->bfield.p[2]); m->cos_pitch = cos(d->bfield.p[2]); }
  int vk = d->vfield.kind;
  if (vk == JSH_V_ACC_PARABOLIC_CONST_CONE || vk == JSH_V_SHEARED_ACC_PARABOLIC_CONST_CONE) {
    double Rz0 = (vk == JSH_V_ACC_PARABOLIC_CONST_CONE) ? d->vfield.p[1] : d->vfield.p[2];
    double z0 = (vk == JSH_V_ACC_PARABOLIC_CONST_CONE) ? d->vfield.p[2] : d->vfield.p[3];
    m->v_cone_oz = (Rz0 * sqrt(z0 / JO_PC) / (0.5 * Rz0 * pow(z0 * JO_PC, -0.5)) - z0);
    m->v_theta = atan(sqrt(Rz0 * Rz0 * z0 / JO_PC) / z0);
  }
  return JSH_OK;
}

static double v_from_gamma(double g) { return JO_C * sqrt(1. - 1. / (g * g)); }

static v3 v_central(double g, v3 o, v3 p) {
  double r = vnorm(vadd(p, o));
  double v_r = JO_C * sqrt(1. - 1. / (g * g));
  return mk(v_r * (p.x + o.x) / r, v_r * (p.y + o.y) / r, v_r * (p.z + o.z) / r);
}

static v3 v_sheared_central(double ga, double gb, double th, v3 o, v3 p) {
  double r = vnorm(vadd(p, o));
  double theta = acos(p.z + o.z / r);
  double g = ga - (ga - gb) * theta / th;
  double v_r = JO_C * sqrt(1. - 1. / (g * g));
  return mk(v_r * (p.x + o.x) / r, v_r * (p.y + o.y) / r, v_r * (p.z + o.z) / r);
}

static v3 v_parabolic_dir(double v_r, double Rz0, v3 p) {
  double r = hypot(p.x, p.y);
  double R = sqrt(Rz0 * Rz0 * p.z / JO_PC);
  double r0 = Rz0 * r / R;
  double alpha = atan(2 * JO_PC * r / r0 / r0);
  if (r == 0) return mk(0, 0, v_r);
  return mk(v_r * cos(alpha) * p.x / r, v_r * cos(alpha) * p.y / r, v_r * sin(alpha));
}

static v3 v_acc_parabolic(double g0, double R0, double Rz0, v3 p) {
  double gamma = 1 + (g0 - 1) / sqrt(R0) * sqrt(p.z);
  return v_parabolic_dir(JO_C * sqrt(1. - 1. / (gamma * gamma)), Rz0, p);
}

static v3 v_sheared_acc_parabolic(double ga0, double gb0, double R0, double Rz0, v3 p) {
  double r = hypot(p.x, p.y);
  double R0_border = sqrt(Rz0 * Rz0 * R0 / JO_PC);
  double R = sqrt(Rz0 * Rz0 * p.z / JO_PC);
  double rR0 = R0_border * r / R;
  double gamma0 = ga0 - (ga0 - gb0) * pow(rR0 / R0_border, 0.25);
  if (gamma0 < 1) gamma0 = 1;
  double gamma = 1 + (gamma0 - 1) / sqrt(R0) * sqrt(p.z);
  return v_parabolic_dir(JO_C * sqrt(1. - 1. / (gamma * gamma)), Rz0, p);
}

static v3 vfield(const model_t* m, v3 p) {
  const double* q = m->d.vfield.p;
  switch (m->d.vfield.kind) {
    case JSH_V_CONST_FLAT: return mk(0, 0, v_from_gamma(q[0]));
    case JSH_V_SHEARED_FLAT: {
      double r = sqrt(p.x * p.x + p.y * p.y);
      double g = q[0] - (q[0] - q[1]) * r / q[2];
      return mk(0, 0, JO_C * sqrt(1. - 1. / (g * g)));
    }
    case JSH_V_SHEATH_FLAT: {
      double r = sqrt(p.x * p.x + p.y * p.y);
      double g = (r < q[2]) ? q[0] : q[1];
      return mk(0, 0, JO_C * sqrt(1. - 1. / (g * g)));
    }
    case JSH_V_CONST_CENTRAL: return v_central(q[0], mk(q[1], q[2], q[3]), p);
    case JSH_V_SHEARED_CENTRAL: return v_sheared_central(q[0], q[1], q[2], mk(q[3], q[4], q[5]), p);
    case JSH_V_SHEATH_CENTRAL: {
      v3 o = mk(q[3], q[4], q[5]);
      double r = vnorm(vadd(p, o));
      double theta = acos(p.z / r);
      double g = (theta < q[2]) ? q[0] : q[1];
      double v_r = JO_C * sqrt(1. - 1. / (g * g));
      return mk(v_r * (p.x + o.x) / r, v_r * (p.y + o.y) / r, v_r * (p.z + o.z) / r);
    }
    case JSH_V_CONST_PARABOLIC: return v_parabolic_dir(JO_C * sqrt(1. - 1. / (q[0] * q[0])), q[1], p);
    case JSH_V_ACC_PARABOLIC: return v_acc_parabolic(q[0], q[1], q[2], p);
    case JSH_V_SHEARED_ACC_PARABOLIC: return v_sheared_acc_parabolic(q[0], q[1], q[2], q[3], p);
    case JSH_V_ACC_PARABOLIC_CONST_CONE:
      if (p.z > q[2]) return v_central(q[0], mk(0, 0, m->v_cone_oz), p);
      return v_acc_parabolic(q[0], q[2], q[1], p);
    case JSH_V_SHEARED_ACC_PARABOLIC_CONST_CONE:
      if (p.z > q[3]) return v_sheared_central(q[0], q[1], m->v_theta, mk(0, 0, m->v_cone_oz), p);
      return v_sheared_acc_parabolic(q[0], q[1], q[3], q[2], p);
    case JSH_V_SIMULATION: {
      double g = sim_value((int32_t)q[0], (int32_t)q[1], p, 1.0);
      return mk(0, 0, JO_C * sqrt(1. - 1. / (g * g)));
    }
    default: return mk(0, 0, 0);
  }
}

static double bscalar(const model_t* m, v3 p) {
  const double* q = m->d.bfield.p;
  switch (m->d.bfield.kind) {
    case JSH_B_RANDOM_SCALAR: return q[0] * pow(vnorm(p) / JO_PC, -q[1]);
    case JSH_B_RANDOM_SCALAR_Z: return q[0] * pow(fabs(p.z) / JO_PC, -q[1]);
    case JSH_B_COMPOSITE_RANDOM_SCALAR_Z: {
      double r = fabs(p.z);
      if (r > q[3]) return q[0] * pow(fabs(p.z) / JO_PC, -q[2]);
      return q[0] * pow(fabs(p.z) / JO_PC, -q[1]);
    }
    default: return 0.0;
  }
}

static v3 bvector(const model_t* m, v3 p) {
  const double* q = m->d.bfield.p;
  switch (m->d.bfield.kind) {
    case JSH_B_CONST_CYLINDER: return mk(0.0, 0.0, q[0] * pow(vnorm(p) / JO_PC, -q[1]));
    case JSH_B_CONST_CYLINDER_Z: return mk(0.0, 0.0, q[0] * pow(fabs(p.z) / JO_PC, -q[1]));
    case JSH_B_RADIAL_CONICAL: {
      double r = vnorm(p);
      return mk(q[0] * pow(r / JO_PC, -q[1]) * p.x / r, q[0] * pow(r / JO_PC, -q[1]) * p.y / r,
                q[0] * pow(r / JO_PC, -q[1]) * p.z / r);
    }
    case JSH_B_TOROIDAL: {
      double fi = atan(p.y / p.x);
      double b = q[0] * pow(p.z / JO_PC, -q[1]);
      return mk(-sin(fi) * b, cos(fi) * b, 0);
    }
    case JSH_B_HELICAL_CYLINDER: {
      double r = sqrt(p.x * p.x + p.y * p.y);
      return mk(q[0] * tan(q[1] * p.y / r), -q[0] * tan(q[1] * p.x / r), q[0]);
    }
    case JSH_B_SPIRAL_CONICAL: {
      double b_z = q[0] / (p.z * p.z / (JO_PC * JO_PC));
      return mk(b_z * (p.x / p.z + p.y * m->tan_pitch / JO_PC), b_z * (p.y / p.z - p.x * m->tan_pitch / JO_PC), b_z);
    }
    case JSH_B_FORCE_FREE_CYLINDRICAL: {
      double fi = atan(p.y / p.x);
      return mk(-q[0] * m->bessel1 * sin(fi), q[0] * m->bessel1 * sin(fi), q[0] * m->bessel0);
    }
    case JSH_B_HELICAL_CONICAL: {
      double b = q[0] * pow(vnorm(p) / JO_PC, -q[1]);
      double rc = sqrt(p.x * p.x + p.y * p.y);
      double px = 0.0, py = 0.0;
      if (rc > 0.0) {
        px = -p.y / rc;
        py = p.x / rc;
        if (q[3] != 0.0 && p.x < 0.0) { px = -px; py = -py; }
      }
      double bt = b * m->sin_pitch;
      return mk(bt * px, bt * py, b * m->cos_pitch);
    }
    case JSH_B_SIMULATION: {
      double fi = atan(p.y / p.x);
      double bp = sim_value((int32_t)q[0], (int32_t)q[1], p, 0.0);
      double bphi = sim_value((int32_t)q[0], (int32_t)q[2], p, 0.0);
      return mk(-sin(fi) * bphi, cos(fi) * bphi, bp);
    }
    default: return mk(0, 0, 0);
  }
}

static double nfield(const model_t* m, v3 p) {
  const double* q = m->d.nfield.p;
  switch (m->d.nfield.kind) {
    case JSH_N_CONST: return q[0];
    case JSH_N_BK: return q[0] * pow(vnorm(p) / JO_PC, -q[1]);
    case JSH_N_BKZ: return q[0] * pow(fabs(p.z) / JO_PC, -q[1]);
    case JSH_N_COMPOSITE_BK: {
      double z = fabs(p.z);
      if (z > q[3]) return q[0] * pow(vnorm(p) / JO_PC, -q[2]);
      return q[0] * pow(vnorm(p) / JO_PC, -q[1]);
    }
    case JSH_N_SIMULATION: return sim_value((int32_t)q[0], (int32_t)q[1], p, 0.0);
    default: return 0.0;
  }
}

/* ====================================================================
 * Lorentz kinematics (src/utils.cpp:147-173) and coefficients
 * (src/utils.cpp:8-144), written as in the reference.
 * ==================================================================== */
static double getG(v3 v) {
  v3 beta = vdiv(v, JO_C);
  return sqrt(1. / (1. - vsq(beta)));
}
static double getD(v3 nl, v3 v) {
  v3 beta = vdiv(v, JO_C);
  return 1. / (getG(v) * (1. - vdot(beta, nl)));
}
static v3 get_n_los_prime(v3 nl, v3 v) {
  double df = getD(nl, v);
  double gamma = getG(v);
  v3 beta = vdiv(v, JO_C);
  return vsub(vmul(nl, df), vmul(beta, (df + 1.) * (gamma / (gamma + 1.))));
}
static v3 getBprime(v3 b, v3 v) {
  double gamma = getG(v);
  double s1 = gamma / ((1. + gamma) * (JO_C * JO_C));
  double vb = vdot(v, b);
  return vadd(vdiv(b, gamma), mk(s1 * v.x * vb, s1 * v.y * vb, s1 * v.z * vb));
}

static double nu_p(double n) { return sqrt(n * JO_Q_E * JO_Q_E / (JO_PI * JO_M_E)); }
static double nu_b_vec(v3 b, v3 nl) { return JO_Q_E * vnorm(vcross(nl, b)) / (2. * JO_PI * JO_M_E * JO_C); }
static double nu_b_scalar(double b) { return JO_Q_E * b / (2. * JO_PI * JO_M_E * JO_C); }
static double nu_b_value(v3 b) { return JO_Q_E * vnorm(b) / (2. * JO_PI * JO_M_E * JO_C); }

enum { CK_I, CK_Q, CK_U, CK_V, CK_F, CK_C, CH_Q, CE_I, CE_Q, CE_U, CE_V, CN };

/* All coefficients at a point in the lab frame: k = k'/D, eta = eta' D D,
 * with the primed quantities from the plasma-frame transforms of
 * Jet::getKI / Jet::getEtaI (src/Jet.cpp:15-46, :218-237). */
/* RandomVectorBField::bf (src/BField.cpp:154-161): b + rnd_fraction |b| n,
 * the wrapper's field taken in the plasma frame (VectorBField(true)). */
static v3 brandom(const model_t* m, v3 b, v3 p, uint32_t k0, uint32_t k1, uint32_t k2) {
  double n[3];
  if (m->d.random.kind == JSH_RND_CELLS) {
    double q[3] = {p.x, p.y, p.z};
    int64_t c = jo_cells_nearest(m->d.random.cells_id, q);
    const double* d = g_cells[m->d.random.cells_id].dir + 3 * (c < 0 ? 0 : c);
    n[0] = d[0]; n[1] = d[1]; n[2] = d[2];
  } else {
    jo_random_direction(m->d.random.seed, k0, k1, k2, n);
  }
  double bv = vnorm(b);
  return vadd(b, vmul(mk(n[0], n[1], n[2]), m->d.random.fraction * bv));
}

static void coefficients_key(const model_t* m, v3 p, v3 nl, double nu, int full, double* k, uint32_t rk0,
                             uint32_t rk1, uint32_t rk2);
static void coefficients(const model_t* m, v3 p, v3 nl, double nu, int full, double* k) {
  coefficients_key(m, p, nl, nu, full, k, 0, 0, 0);
}

/* (rk0, rk1, rk2): pixel, frequency and evaluation index of the per-
 * evaluation random direction (JSH_RND_POINTS). */
static void coefficients_key(const model_t* m, v3 p, v3 nl, double nu, int full, double* k, uint32_t rk0,
                             uint32_t rk1, uint32_t rk2) {
  v3 v = vfield(m, p);
  double gamma = getG(v);
  double D = getD(nl, v);
  double n = nfield(m, p);
  double n_prime = m->d.nfield.in_plasma_frame ? n : n / gamma;
  double nu_prime = nu / D;
  double s = m->d.s;
  for (int i = 0; i < CN; ++i) k[i] = 0.0;
  if (m->b_scalar) {
    double b = bscalar(m, p);
    double np = nu_p(n_prime);
    double nb = nu_b_scalar(b);
    double k0 = JO_PI * np * np * nb / (JO_C * nu_prime * nu_prime);
    double ki = k0 * pow(nb / nu_prime, s / 2.) * (m->fk_i * m->rnd_k);
    double e0 = JO_PI * np * np * nb * JO_M_E / JO_C;
    double ei = e0 * pow(nb / nu_prime, (s - 1.) / 2.) * (m->fe_i * m->rnd_e);
    k[CK_I] = ki / D;
    k[CE_I] = ei * D * D;
    return;
  }
  v3 bl = bvector(m, p);
  int rnd = m->d.random.kind != JSH_RND_NONE;
  if (rnd) bl = brandom(m, bl, p, rk0, rk1, rk2);
  v3 b = (m->d.bfield.in_plasma_frame || rnd) ? bl : getBprime(bl, v);
  v3 nlp = get_n_los_prime(nl, v);
  double np = nu_p(n_prime);
  double nb = nu_b_vec(b, nlp);
  double k0 = JO_PI * np * np * nb / (JO_C * nu_prime * nu_prime);
  double ki = k0 * pow(nb / nu_prime, s / 2.) * m->fk_i;
  double e0 = JO_PI * np * np * nb * JO_M_E / JO_C;
  double ei = e0 * pow(nb / nu_prime, (s - 1.) / 2.) * m->fe_i;
  k[CK_I] = ki / D;
  k[CE_I] = ei * D * D;
  if (!full) return;
  double cos_theta = vdot(b, nlp) / vnorm(b);
  double nbv = nu_b_value(b);
  double k0v = JO_PI * np * np * nbv / (JO_C * nu_prime * nu_prime);
  double kv = -k0v * cos_theta * pow(nb / nu_prime, (s + 1.) / 2.) * m->fk_v;
  double kfc = 2. * JO_PI * np * np * nbv * cos_theta / (JO_C * nu_prime * nu_prime);
  double kcc = -JO_PI * np * np * nb * nb / (JO_C * nu_prime * nu_prime * nu_prime);
  double kf = m->kfr_factor * kfc;
  double kc = m->kcr_a * (m->kcr_b - pow(nb / nu_prime, (s - 2.) / 2.)) * kcc;
  if (m->d.thermal_fraction != 0.0) {
    double npt = nu_p(m->d.thermal_fraction * n_prime);
    kf = kf + 2. * JO_PI * npt * npt * nbv * cos_theta / (JO_C * nu_prime * nu_prime);
    kc = kc + -JO_PI * npt * npt * nb * nb / (JO_C * nu_prime * nu_prime * nu_prime);
  }
  double e0v = JO_PI * np * np * nbv * JO_M_E / JO_C;
  double ev = -e0v * cos_theta * pow(nb / nu_prime, s / 2.) * m->fe_v;
  k[CK_Q] = (m->kq_ratio * ki) / D;
  k[CK_V] = kv / D;
  k[CK_F] = kf / D;
  k[CK_C] = kc / D;
  k[CE_Q] = (m->eq_ratio * ei) * D * D;
  k[CE_V] = ev * D * D;
}

int jo_coefficients(const jsh_model_desc* model, const double* point, const double* n_los, double nu,
                    double* out) {
  model_t m;
  int st = model_init(model, &m);
  if (st) return st;
  coefficients(&m, mk(point[0], point[1], point[2]), mk(n_los[0], n_los[1], n_los[2]), nu, 1, out);
  return JSH_OK;
}

/* The field laws at a lab-frame point [cm]: out = {B (the vector; a scalar
 * law's |B| in out[0], 0, 0), n, v (3) [cm/s]} (BField::bf, NField::nf,
 * VField::vf of src/BField.cpp, src/NField.cpp, src/VField.cpp); for the
 * known-answer tests of the laws. */
int jo_fields(const jsh_model_desc* model, const double* point, double* out) {
  model_t m;
  int st = model_init(model, &m);
  if (st) return st;
  const v3 p = mk(point[0], point[1], point[2]);
  if (m.b_scalar) {
    out[0] = bscalar(&m, p);
    out[1] = out[2] = 0.0;
  } else {
    const v3 b = bvector(&m, p);
    out[0] = b.x;
    out[1] = b.y;
    out[2] = b.z;
  }
  out[3] = nfield(&m, p);
  const v3 v = vfield(&m, p);
  out[4] = v.x;
  out[5] = v.y;
  out[6] = v.z;
  return JSH_OK;
}

/* ====================================================================
 * Dormand-Prince 5(4) with dense output and odeint-documented control.
 * ==================================================================== */
static const double DP_C2 = 1.0 / 5, DP_C3 = 3.0 / 10, DP_C4 = 4.0 / 5, DP_C5 = 8.0 / 9;
static const double DP_A21 = 1.0 / 5;
static const double DP_A31 = 3.0 / 40, DP_A32 = 9.0 / 40;
static const double DP_A41 = 44.0 / 45, DP_A42 = -56.0 / 15, DP_A43 = 32.0 / 9;
static const double DP_A51 = 19372.0 / 6561, DP_A52 = -25360.0 / 2187, DP_A53 = 64448.0 / 6561, DP_A54 = -212.0 / 729;
static const double DP_A61 = 9017.0 / 3168, DP_A62 = -355.0 / 33, DP_A63 = 46732.0 / 5247, DP_A64 = 49.0 / 176,
                    DP_A65 = -5103.0 / 18656;
static const double DP_B1 = 35.0 / 384, DP_B3 = 500.0 / 1113, DP_B4 = 125.0 / 192, DP_B5 = -2187.0 / 6784,
                    DP_B6 = 11.0 / 84;
static const double DP_E1 = 71.0 / 57600, DP_E3 = -71.0 / 16695, DP_E4 = 71.0 / 1920, DP_E5 = -17253.0 / 339200,
                    DP_E6 = 22.0 / 525, DP_E7 = -1.0 / 40;
static const double DP_D1 = -12715105075.0 / 11282082432.0, DP_D3 = 87487479700.0 / 32700410799.0,
                    DP_D4 = -10690763975.0 / 1880347072.0, DP_D5 = 701980252875.0 / 199316789632.0,
                    DP_D6 = -1453857185.0 / 822651844.0, DP_D7 = 69997945.0 / 29380423.0;

#define NS 4 /* state width: tau uses component 0, IQUV all four */

typedef void (*rhs_fn)(void* ctx, double t, const double* x, double* dxdt);

typedef struct {
  rhs_fn f;
  void* ctx;
  int dim;
  uint64_t evals;
} sys_t;

static void sys_eval(sys_t* S, double t, const double* x, double* dx) {
  S->f(S->ctx, t, x, dx);
  S->evals++;
}

/* One Dormand-Prince step.  k[0] = f(t, x) on entry; on return x_new,
 * k[1..6] the stages (k[6] = f(t + dt, x_new), FSAL) and err. */
static void dp_step(sys_t* S, double t, const double* x, double dt, double k[7][NS], double* xn, double* err) {
  int n = S->dim;
  double y[NS] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i) y[i] = x[i] + dt * (DP_A21 * k[0][i]);
  sys_eval(S, t + DP_C2 * dt, y, k[1]);
  for (int i = 0; i < n; ++i) y[i] = x[i] + dt * (DP_A31 * k[0][i] + DP_A32 * k[1][i]);
  sys_eval(S, t + DP_C3 * dt, y, k[2]);
  for (int i = 0; i < n; ++i) y[i] = x[i] + dt * (DP_A41 * k[0][i] + DP_A42 * k[1][i] + DP_A43 * k[2][i]);
  sys_eval(S, t + DP_C4 * dt, y, k[3]);
  for (int i = 0; i < n; ++i)
    y[i] = x[i] + dt * (DP_A51 * k[0][i] + DP_A52 * k[1][i] + DP_A53 * k[2][i] + DP_A54 * k[3][i]);
  sys_eval(S, t + DP_C5 * dt, y, k[4]);
  for (int i = 0; i < n; ++i)
    y[i] = x[i] + dt * (DP_A61 * k[0][i] + DP_A62 * k[1][i] + DP_A63 * k[2][i] + DP_A64 * k[3][i] +
                        DP_A65 * k[4][i]);
  sys_eval(S, t + dt, y, k[5]);
  for (int i = 0; i < n; ++i)
    xn[i] = x[i] + dt * (DP_B1 * k[0][i] + DP_B3 * k[2][i] + DP_B4 * k[3][i] + DP_B5 * k[4][i] + DP_B6 * k[5][i]);
  sys_eval(S, t + dt, xn, k[6]);
  for (int i = 0; i < n; ++i)
    err[i] = dt * (DP_E1 * k[0][i] + DP_E3 * k[2][i] + DP_E4 * k[3][i] + DP_E5 * k[4][i] + DP_E6 * k[5][i] +
                   DP_E7 * k[6][i]);
}

/* odeint default_error_checker: max_i |err_i| / (atol + rtol (|x_i| + |dt| |dxdt_i|)) */
static double err_norm(int n, const double* err, const double* x, const double* dxdt, double dt, double atol,
                       double rtol) {
  double m = 0.0;
  for (int i = 0; i < n; ++i) {
    double e = fabs(err[i]) / (atol + rtol * (fabs(x[i]) + fabs(dt) * fabs(dxdt[i])));
    if (isnan(e)) return e;
    if (e > m) m = e;
  }
  return m;
}

static double dt_decrease(double dt, double err, double max_dt) {
  double f = 0.9 * pow(err, -1.0 / 3.0);
  dt *= (f > 0.2 ? f : 0.2);
  if (max_dt != 0.0 && fabs(dt) > max_dt) dt = max_dt;
  return dt;
}

static double dt_increase(double dt, double err, double max_dt) {
  if (err < 0.5) {
    double e = err > pow(5.0, -5.0) ? err : pow(5.0, -5.0);
    dt *= 9.0 / 10.0 * pow(e, -1.0 / 5.0);
    if (max_dt != 0.0 && fabs(dt) > max_dt) dt = max_dt;
  }
  return dt;
}

/* Dense output of the last step at t in [t_old, t_old + dt]. */
/* k1 is the first stage of that step; k[2..6] its stages 3..7. */
static void dp_dense(int n, double t_old, double dt, const double* x_old, const double* x_new, const double* k1,
                     double k[7][NS], double t, double* out) {
  double theta = (t - t_old) / dt;
  double th1 = 1.0 - theta;
  for (int i = 0; i < n; ++i) {
    double ydiff = x_new[i] - x_old[i];
    double bspl = dt * k1[i] - ydiff;
    double r4 = ydiff - dt * k[6][i] - bspl;
    double r5 = dt * (DP_D1 * k1[i] + DP_D3 * k[2][i] + DP_D4 * k[3][i] + DP_D5 * k[4][i] + DP_D6 * k[5][i] +
                      DP_D7 * k[6][i]);
    out[i] = x_old[i] + theta * (ydiff + th1 * (bspl + theta * (r4 + th1 * r5)));
  }
}

typedef struct {
  double atol, rtol, max_dt;
  int64_t max_steps;
  uint64_t acc, rej;
  uint32_t status;
} ctl_t;

#define FAIL_LIMIT 500

/* One successful controlled step (retrying rejected attempts), odeint
 * controlled_runge_kutta::try_step semantics with the FSAL derivative in
 * k[0].  Returns 0 on success, else a status bit. */
static uint32_t controlled_step(sys_t* S, ctl_t* C, double* t, double* x, double* dt, double k[7][NS],
                                double* x_old_out, double* k1_old, double* dt_used, int64_t* nsteps) {
  int n = S->dim;
  int fails = 0;
  for (;;) {
    if ((*nsteps)++ >= C->max_steps) return JSH_ST_STEP_LIMIT;
    if (C->max_dt != 0.0 && fabs(*dt) > C->max_dt) {
      *dt = C->max_dt;
      C->rej++;
      if (++fails >= FAIL_LIMIT) return JSH_ST_FAIL_LIMIT;
      continue;
    }
    double xn[NS], err[NS];
    dp_step(S, *t, x, *dt, k, xn, err);
    double e = err_norm(n, err, x, k[0], *dt, C->atol, C->rtol);
    if (e != e) return JSH_ST_NAN;
    if (e > 1.0) {
      *dt = dt_decrease(*dt, e, C->max_dt);
      C->rej++;
      if (++fails >= FAIL_LIMIT) return JSH_ST_FAIL_LIMIT;
      continue;
    }
    double t_new = *t + *dt;
    if (t_new == *t) return JSH_ST_DT_UNDERFLOW;
    for (int i = 0; i < n; ++i) { x_old_out[i] = x[i]; x[i] = xn[i]; }
    *dt_used = *dt;
    *t = t_new;
    *dt = dt_increase(*dt, e, C->max_dt);
    for (int i = 0; i < n; ++i) { k1_old[i] = k[0][i]; k[0][i] = k[6][i]; }
    C->acc++;
    return 0;
  }
}

/* ====================================================================
 * The per-pixel transfer (src/Observation.cpp:126-214, :242-308, :349-395).
 * ==================================================================== */
typedef struct {
  const model_t* m;
  v3 p0, dir;   /* point(t) = p0 + t dir */
  v3 nl;        /* LOS unit vector towards the observer */
  double nu;
  int full;
  uint32_t rk0, rk1;  /* random-direction key of the item: pixel, frequency */
  uint32_t* ev;       /* the item's evaluation counter */
} tctx_t;

static void rhs_tau(void* c, double t, const double* x, double* dx) {
  (void)x;
  tctx_t* T = (tctx_t*)c;
  v3 p = vadd(T->p0, vmul(T->dir, t));
  double k[CN];
  coefficients_key(T->m, p, T->nl, T->nu, 0, k, T->rk0, T->rk1, T->ev ? (*T->ev)++ : 0u);
  dx[0] = k[CK_I];
}

static void rhs_iquv(void* c, double t, const double* x, double* dx) {
  tctx_t* T = (tctx_t*)c;
  v3 p = vadd(T->p0, vmul(T->dir, t));
  double k[CN];
  coefficients_key(T->m, p, T->nl, T->nu, T->full, k, T->rk0, T->rk1, T->ev ? (*T->ev)++ : 0u);
  if (!T->full) {
    dx[0] = k[CE_I] - k[CK_I] * x[0];
    return;
  }
  dx[0] = k[CE_I] - k[CK_I] * x[0] - k[CK_Q] * x[1] - k[CK_U] * x[2] - k[CK_V] * x[3];
  dx[1] = k[CE_Q] - k[CK_I] * x[1] - k[CK_Q] * x[0] - k[CK_F] * x[2] - k[CH_Q] * x[3];
  dx[2] = k[CE_U] - k[CK_I] * x[2] - k[CK_U] * x[0] + k[CK_F] * x[1] - k[CK_C] * x[3];
  dx[3] = k[CE_V] - k[CK_I] * x[3] - k[CK_V] * x[0] + k[CH_Q] * x[1] + k[CK_C] * x[2];
}

/* steps_schedule (src/utils.cpp:354-366) with its default tau limits. */
static int steps_schedule(double tau, int n_min, int n_max) {
  double tau_min = 0.1, tau_max = 100.0;
  if (tau <= tau_min) return n_min;
  if (tau >= tau_max) return n_max;
  double b = -log(tau_min);
  double k = n_max / pow((log(tau_max) + b), 2.0);
  double n = k * pow((log(tau) + b), 2.0) + n_min;
  return (int)ceil(n);
}

int jo_steps_schedule(double tau, int n_min, int n_max) { return steps_schedule(tau, n_min, n_max); }

typedef struct {
  double tau, l, iquv[4];
  uint32_t status;
} pix_out_t;

static void render_ray(const model_t* m, v3 ro, v3 rd, v3 rd_renorm, double nu, const jsh_params* P,
                       pix_out_t* o, jo_counters* cnt, uint32_t pix, uint32_t f) {
  uint32_t ev = 0; /* evaluation index of the item (random-direction key) */
  memset(o, 0, sizeof(*o));
  hits_t h;
  geo_hit(&m->geo, ro, rd, &h);
  o->status = h.status;
  if (h.n == 0) return;
  o->status |= JSH_ST_HIT;
  int64_t max_steps = P->max_steps > 0 ? P->max_steps : ((int64_t)1 << 22);
  v3 nl = vmul(rd, -1.);
  int full = (P->output == JSH_OUT_FULL);

  /* ---- tau pass: front to back, dense output, stop at tau_max ---- */
  double background_tau = 0.0, thickness = 0.0;
  int nseg = h.n;
  for (int sidx = 0; sidx < nseg; ++sidx) {
    v3 pin = h.s[sidx].in, pout = h.s[sidx].out;
    double length = vnorm(vsub(pout, pin));
    double dt = length / P->n;
    tctx_t T = {m, pin, rd, nl, nu, 0, pix, f, &ev};
    sys_t S = {rhs_tau, &T, 1, 0};
    ctl_t C = {P->tau_atol, P->tau_rtol, P->dt_max, max_steps, 0, 0, 0};
    double t = 0.0, x[NS] = {0, 0, 0, 0}, k[7][NS], x_old[NS] = {0}, k1_old[NS] = {0}, dt_used = 0.0, t_old = 0.0;
    int deriv_init = 0, crossed = 0;
    int64_t nsteps = 0;
    uint32_t fail = 0;
    /* adaptive_iterator: advance while t < t_end (odeint less_with_sign) */
    while (length - t > DBL_EPSILON) {
      if ((t + dt) - length > DBL_EPSILON) dt = length - t; /* end exactly at t_end */
      if (!deriv_init) { sys_eval(&S, t, x, k[0]); deriv_init = 1; }
      t_old = t;
      fail = controlled_step(&S, &C, &t, x, &dt, k, x_old, k1_old, &dt_used, &nsteps);
      if (fail) break;
      if (x[0] >= P->tau_max) { crossed = 1; break; }
    }
    cnt->rhs_evals += S.evals;
    cnt->steps_accepted += C.acc;
    cnt->steps_rejected += C.rej;
    if (fail) { o->status |= fail; o->tau = background_tau + x[0]; o->l = thickness + length; return; }
    if (crossed) {
      /* bisection on the dense output of the crossing step */
      o->status |= JSH_ST_TAU_CROSSED;
      double t0 = t_old, t1 = t, xm[NS], t_m;
      xm[0] = x[0];
      int it = 0;
      while (fabs(xm[0] - P->tau_max) > P->tau_precision) {
        if (++it > 200) { o->status |= JSH_ST_BISECT_LIMIT; break; }
        t_m = 0.5 * (t0 + t1);
        dp_dense(1, t_old, dt_used, x_old, x, k1_old, k, t_m, xm);
        if (xm[0] > P->tau_max) t1 = t_m;
        else t0 = t_m;
      }
      t_m = 0.5 * (t0 + t1);
      /* Ray(point_in, ray_direction).point(t_m): the Ray ctor re-normalises */
      h.s[sidx].out = ray_point(pin, rd_renorm, t_m);
      nseg = sidx + 1;
    }
    background_tau += x[0];
    thickness += length;
    if (crossed) break;
  }
  o->tau = background_tau;
  o->l = thickness;
  if (!(background_tau > P->tau_min)) return;
  o->status |= JSH_ST_IQUV;

  /* ---- I / IQUV pass: back to front, controlled stepper ---- */
  double st[NS] = {0, 0, 0, 0};
  int dim = full ? 4 : 1;
  for (int sidx = nseg - 1; sidx >= 0; --sidx) {
    v3 pin = h.s[sidx].in, pout = h.s[sidx].out;
    double length = vnorm(vsub(pout, pin));
    double auto_n = P->n;
    if (background_tau > 0.1) auto_n = steps_schedule(background_tau, P->n, 10 * P->n);
    double dt = length / auto_n;
    tctx_t T = {m, pout, nl, nl, nu, full, pix, f, &ev};
    sys_t S = {rhs_iquv, &T, dim, 0};
    ctl_t C = {P->atol, P->rtol, 0.0, max_steps, 0, 0, 0};
    double t = 0.0, k[7][NS], x_old[NS], k1_old[NS], dt_used;
    int64_t nsteps = 0;
    uint32_t fail = 0;
    int first = 1;
    while (length - t > DBL_EPSILON) {
      if ((t + dt) - length > DBL_EPSILON) dt = length - t;
      if (first) { sys_eval(&S, t, st, k[0]); first = 0; }
      fail = controlled_step(&S, &C, &t, st, &dt, k, x_old, k1_old, &dt_used, &nsteps);
      if (fail) break;
    }
    cnt->rhs_evals += S.evals;
    cnt->steps_accepted += C.acc;
    cnt->steps_rejected += C.rej;
    if (fail) { o->status |= fail; break; }
  }
  for (int i = 0; i < 4; ++i) o->iquv[i] = st[i];
}

/* Optional per-item RHS evaluation counts of the next renders ([n_nu][n_sel]). */
static uint64_t* g_item_evals = NULL;
void jo_set_item_evals(uint64_t* buf) { g_item_evals = buf; }

int jo_render(const jsh_model_desc* model, const jsh_plane_desc* plane, const double* nu, int32_t n_nu,
              const jsh_params* params, const int64_t* pix_idx, int64_t n_sel, int32_t n_threads, jsh_image* out,
              jo_counters* counters) {
  if (!model || !plane || !nu || n_nu < 1 || !params || !out) return JSH_ERR_INVALID;
  if (params->n < 1 || !(params->tau_max > 0)) return JSH_ERR_INVALID;
  model_t m;
  int st = model_init(model, &m);
  if (st) return st;
  plane_t p;
  st = plane_build(plane, &p);
  if (st) return st;
  int64_t npix = (int64_t)(p.n_across * p.n_along);
  if (!pix_idx) n_sel = npix;
  v3 rd = p.dir;
  v3 rd2 = vnormalize(rd);
  uint64_t tot_evals = 0, tot_acc = 0, tot_rej = 0;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
  int64_t nwork = n_sel * (int64_t)n_nu;
#pragma omp parallel for schedule(dynamic) reduction(+ : tot_evals, tot_acc, tot_rej)
  for (int64_t w = 0; w < nwork; ++w) {
    int64_t sel = w / n_nu;
    int f = (int)(w % n_nu);
    int64_t pix = pix_idx ? pix_idx[sel] : sel;
    v3 ro = plane_origin(&p, (uint64_t)pix / p.n_along, (uint64_t)pix % p.n_along);
    pix_out_t o;
    jo_counters c = {0, 0, 0};
    render_ray(&m, ro, rd, rd2, nu[f], params, &o, &c, (uint32_t)pix, (uint32_t)f);
    int64_t q = (int64_t)f * n_sel + sel;
    if (out->tau) out->tau[q] = o.tau;
    if (out->l) out->l[q] = o.l;
    if (out->I) out->I[q] = o.iquv[0];
    if (out->Q) out->Q[q] = o.iquv[1];
    if (out->U) out->U[q] = o.iquv[2];
    if (out->V) out->V[q] = o.iquv[3];
    if (out->status) out->status[q] = o.status;
    if (g_item_evals) g_item_evals[q] = c.rhs_evals;
    tot_evals += c.rhs_evals;
    tot_acc += c.steps_accepted;
    tot_rej += c.steps_rejected;
  }
  if (counters) {
    counters->rhs_evals = tot_evals;
    counters->steps_accepted = tot_acc;
    counters->steps_rejected = tot_rej;
  }
  plane_free(&p);
  return JSH_OK;
}

/* ====================================================================
 * Stripe mode: Observation::run_stripe (src/Observation.cpp:310-347) with
 * integrate_tau (src/Observation.cpp:55-123) and Image::getStripe
 * (src/Image.cpp:31-41).  Tau only, for the pixels of row n_across / 2 from
 * column n_along / 2 to the end; per intersection a constant-step
 * classical RK4 (odeint runge_kutta4) over the const-step time range
 * [0, L] with dt = L / n, stopped at the first yielded state with tau >=
 * tau_max (that state's tau is kept and later intersections are dropped);
 * otherwise the state after the last step.  odeint's const-step iterator
 * steps while (t + dt) - L <= DBL_EPSILON with t = step * dt.  Pixels whose
 * ray misses keep tau = 0.
 * ==================================================================== */
static double stripe_ray(const model_t* m, v3 ro, v3 rd, double nu, int n, double tau_max) {
  hits_t h;
  geo_hit(&m->geo, ro, rd, &h);
  v3 nl = vmul(rd, -1.);
  double bg = 0.0;
  for (int sidx = 0; sidx < h.n; ++sidx) {
    v3 pin = h.s[sidx].in, pout = h.s[sidx].out;
    double length = vnorm(vsub(pout, pin));
    double dt = length / n;
    tctx_t T = {m, pin, rd, nl, nu, 0, 0, 0, NULL};
    double x = 0.0, t = 0.0, k1, k2, k4, dum = 0.0;
    int64_t step = 0;
    int found = (x >= tau_max);
    if (dt > 0.0) {
      const double w1 = (1.0 / 6.0) * dt, w2 = (1.0 / 3.0) * dt;
      while (!found && (t + dt) - length <= DBL_EPSILON && step <= (int64_t)n + 1) {
        rhs_tau(&T, t, &dum, &k1);
        rhs_tau(&T, t + 0.5 * dt, &dum, &k2); /* k3 = k2: dtau/dt does not depend on tau */
        rhs_tau(&T, t + dt, &dum, &k4);
        x = (((x + w1 * k1) + w2 * k2) + w2 * k2) + w1 * k4;
        ++step;
        t = (double)step * dt;
        found = (x >= tau_max);
      }
    }
    bg += x;
    if (found) break;
  }
  return bg;
}

int jo_stripe(const jsh_model_desc* model, const jsh_plane_desc* plane, double nu, int32_t n, double tau_max,
              double* tau_out) {
  if (!model || !plane || !tau_out || n < 1 || !(nu > 0)) return JSH_ERR_INVALID;
  model_t m;
  int st = model_init(model, &m);
  if (st) return st;
  plane_t p;
  st = plane_build(plane, &p);
  if (st) return st;
  const uint64_t row = p.n_across / 2, c0 = p.n_along / 2;
  const int64_t count = (int64_t)(p.n_along - c0);
#pragma omp parallel for schedule(dynamic)
  for (int64_t i = 0; i < count; ++i) {
    v3 ro = plane_origin(&p, row, c0 + (uint64_t)i);
    tau_out[i] = stripe_ray(&m, ro, p.dir, nu, n, tau_max);
  }
  plane_free(&p);
  return JSH_OK;
}

/* ====================================================================
 * Integrator known-answer hooks.
 * ==================================================================== */
typedef struct { double a, b; } lin_t;
static void rhs_lin(void* c, double t, const double* x, double* dx) {
  (void)t;
  lin_t* L = (lin_t*)c;
  dx[0] = L->a * x[0] + L->b;
}

double jo_test_linear_dense(double a, double b, double L, double dt0, double atol, double rtol, int64_t* n_steps) {
  lin_t lc = {a, b};
  sys_t S = {rhs_lin, &lc, 1, 0};
  ctl_t C = {atol, rtol, 0.0, (int64_t)1 << 30, 0, 0, 0};
  double t = 0.0, x[NS] = {0}, k[7][NS], x_old[NS], k1_old[NS], dt = dt0, dt_used;
  int64_t ns = 0;
  int init = 0;
  while (L - t > DBL_EPSILON) {
    if ((t + dt) - L > DBL_EPSILON) dt = L - t;
    if (!init) { sys_eval(&S, t, x, k[0]); init = 1; }
    if (controlled_step(&S, &C, &t, x, &dt, k, x_old, k1_old, &dt_used, &ns)) break;
  }
  if (n_steps) *n_steps = (int64_t)C.acc;
  return x[0];
}

double jo_test_linear_controlled(double a, double b, double L, double dt0, double atol, double rtol,
                                 int64_t* n_steps) {
  return jo_test_linear_dense(a, b, L, dt0, atol, rtol, n_steps);
}

static void rhs_exp(void* c, double t, const double* x, double* dx) {
  (void)c; (void)t;
  dx[0] = x[0];
}

double jo_test_dense_error(double h, double theta) {
  sys_t S = {rhs_exp, NULL, 1, 0};
  double x[NS] = {1.0}, k[7][NS], xn[NS], err[NS], out[NS];
  sys_eval(&S, 0.0, x, k[0]);
  dp_step(&S, 0.0, x, h, k, xn, err);
  dp_dense(1, 0.0, h, x, xn, k[0], k, theta * h, out);
  return out[0] - exp(theta * h);
}

/* ====================================================================
 * Cosmology: comoving_transfer_distance2 + mas_to_pc (src/utils.cpp:186-208,
 * :373-378): dx/dt = ((Om + (1+t) g_nu)(1+t)^3 + OV)^-1/2, integrated from 0
 * to z with the controlled stepper at atol = rtol = 1.49e-8, dt0 = 1e-9.
 * ==================================================================== */
typedef struct { double om, ov, gnu; } ctd_t;
static void rhs_ctd(void* c, double t, const double* x, double* dx) {
  (void)x;
  ctd_t* q = (ctd_t*)c;
  dx[0] = pow((q->om + (1. + t) * q->gnu) * (1. + t) * (1. + t) * (1. + t) + q->ov, -0.5);
}

double jo_mas_to_pc(double z, const jsh_cosmology* cosmo) {
  jsh_cosmology dflt = {69.32, 0.2865, 0.7134130719051658, 8.69280948342326e-05};
  if (!cosmo) cosmo = &dflt;
  ctd_t q = {cosmo->omega_M, cosmo->omega_V, cosmo->gamma_nu};
  sys_t S = {rhs_ctd, &q, 1, 0};
  ctl_t C = {1.49e-8, 1.49e-8, 0.0, (int64_t)1 << 30, 0, 0, 0};
  double t = 0.0, x[NS] = {0}, k[7][NS], x_old[NS], k1_old[NS], dt = 1E-09, dt_used;
  int64_t ns = 0;
  int init = 0;
  while (z - t > DBL_EPSILON) {
    if ((t + dt) - z > DBL_EPSILON) dt = z - t;
    if (!init) { sys_eval(&S, t, x, k[0]); init = 1; }
    if (controlled_step(&S, &C, &t, x, &dt, k, x_old, k1_old, &dt_used, &ns)) break;
  }
  double ctd = (299792.458 / cosmo->H0) * pow(10., 6.) * x[0];
  double d_a = ctd / (1. + z);
  return JO_MAS_TO_RAD * d_a;
}

int jo_openmp_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
