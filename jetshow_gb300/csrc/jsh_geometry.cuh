// jsh_geometry.cuh -- FP64 ray generation and ray/jet intersection on the
// device.  Every floating-point operation is an explicit round-to-nearest
// intrinsic (__dadd_rn, __dmul_rn, __ddiv_rn, __dsqrt_rn) so nvcc cannot
// contract anything into an FMA; with the host-precomputed constants of
// JshModel / JshPlane this makes the hit mask and the segment end points
// bit-exact with the oracle, whose C code fixes the same evaluation order.
//
// Reference: src/Cone.cpp:48-118, src/Geometry.cpp:28-78,
// src/Cylinder.cpp:29-99, src/Parabaloid.cpp:39-60,
// src/ParabaloidCone.cpp:36-94, src/Intersection.cpp:41-62,
// src/Geometry.cpp:92-132 (SimulationGeometry),
// src/Image.cpp:44-194, src/ImagePlane.cpp:11-33.
#pragma once

#include "jsh_model.h"

namespace jsh {

struct V3 {
  double x, y, z;
};

__device__ __forceinline__ double ad(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sb(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double sq(double a) { return __dsqrt_rn(a); }

__device__ __forceinline__ V3 mk(double x, double y, double z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return mk(ad(a.x, b.x), ad(a.y, b.y), ad(a.z, b.z)); }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return mk(sb(a.x, b.x), sb(a.y, b.y), sb(a.z, b.z)); }
__device__ __forceinline__ V3 vmul(V3 a, double s) { return mk(ml(a.x, s), ml(a.y, s), ml(a.z, s)); }
__device__ __forceinline__ V3 vdiv(V3 a, double s) { return mk(dv(a.x, s), dv(a.y, s), dv(a.z, s)); }
// (a0 b0 + a1 b1) + a2 b2
__device__ __forceinline__ double vdot(V3 a, V3 b) { return ad(ad(ml(a.x, b.x), ml(a.y, b.y)), ml(a.z, b.z)); }
__device__ __forceinline__ double vsq(V3 a) { return vdot(a, a); }
__device__ __forceinline__ double vnorm(V3 a) { return sq(vsq(a)); }
__device__ __forceinline__ V3 vnormalize(V3 a) {
  double n = vsq(a);
  if (n > 0.0) return vdiv(a, sq(n));
  return a;
}
__device__ __forceinline__ V3 ray_point(V3 o, V3 d, double t) { return vadd(o, vmul(d, t)); }

struct Seg {
  V3 in, out;
};
struct Hits {
  int n;
  uint32_t status;
  Seg s[JSH_MAX_SEG];
};

// ---------------------------------------------------------------- plane
// Ray origin of pixel (row i across, column j along); see the oracle's
// plane_origin for the layout of the across table.
__device__ __forceinline__ V3 plane_origin(const JshPlane& p, uint64_t i, uint64_t j) {
  uint64_t nh = p.n_across / 2;
  double across;
  if (i < nh) across = p.across_pos[(nh - i - 1) * p.n_along + j];
  else across = -p.across_pos[(i - nh) * p.n_along + j];
  return mk(ml(1., 0.0), ml(1., across), ml(p.inv_sin, p.along_center[j]));
}

// ---------------------------------------------------------------- cone
__device__ __forceinline__ Seg full_infinite(V3 ro, V3 rd, V3 go, double big_scale) {
  V3 diff = vsub(ro, go);
  V3 ref = vsub(diff, vmul(rd, vdot(diff, rd)));
  return Seg{vsub(ref, vmul(rd, big_scale)), vadd(ref, vmul(rd, big_scale))};
}

__device__ __forceinline__ bool cone_is_within(const JshCone& c, V3 p) {
  V3 diff = vnormalize(vsub(p, mk(c.ox, c.oy, c.oz)));
  double cosp = vdot(mk(c.dx, c.dy, c.dz), diff);
  return cosp > c.cos_angle || cosp < -c.cos_angle;
}

__device__ __forceinline__ Seg cone_half_infinite(const JshCone& c, V3 rd, V3 point) {
  V3 check = vsub(point, rd);
  if (cone_is_within(c, check)) return Seg{vsub(point, vmul(rd, c.big_scale)), point};
  return Seg{point, vadd(point, vmul(rd, c.big_scale))};
}

__device__ __forceinline__ void cone_hit(const JshCone& c, V3 ro, V3 rd, Hits& h) {
  h.n = 0;
  V3 delta = vsub(ro, mk(c.ox, c.oy, c.oz));
  double cos2 = ml(c.cos_angle, c.cos_angle);
  const double d[3] = {c.dx, c.dy, c.dz};
  double M[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) M[i][j] = sb(ml(d[i], d[j]), ml(cos2, i == j ? 1.0 : 0.0));
  const double r[3] = {rd.x, rd.y, rd.z}, e[3] = {delta.x, delta.y, delta.z};
  double u[3], w[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    u[j] = ad(ad(ml(r[0], M[0][j]), ml(r[1], M[1][j])), ml(r[2], M[2][j]));
    w[j] = ad(ad(ml(e[0], M[0][j]), ml(e[1], M[1][j])), ml(e[2], M[2][j]));
  }
  double c2 = ad(ad(ml(u[0], r[0]), ml(u[1], r[1])), ml(u[2], r[2]));
  double c1 = ad(ad(ml(u[0], e[0]), ml(u[1], e[1])), ml(u[2], e[2]));
  double c0 = ad(ad(ml(w[0], e[0]), ml(w[1], e[1])), ml(w[2], e[2]));
  double disc = sb(ml(c1, c1), ml(c0, c2));
  if (disc < 0) return;
  if (disc == 0) {
    double t = dv(-c1, c2);
    V3 point = ray_point(ro, rd, t);
    V3 dp = vsub(point, mk(c.ox, c.oy, c.oz));
    double lim = ml(1E-06, 1E-06);
    h.n = 1;
    if (vsq(dp) <= ml(lim, lim) && c1 == 0.0) {
      h.s[0] = full_infinite(ro, rd, mk(c.ox, c.oy, c.oz), c.big_scale);
    } else {
      h.s[0] = Seg{point, point};
    }
    return;
  }
  double eps = (c1 > 0 ? 1 : -1);
  double root = sq(sb(ml(c1, c1), ml(c2, c0)));
  double den = sb(-c1, ml(eps, root));
  double t1 = dv(den, c2);
  double t2 = dv(c0, den);
  V3 pin = ray_point(ro, rd, fmin(t1, t2));
  V3 pout = ray_point(ro, rd, fmax(t1, t2));
  double cos_ray_cone = vdot(rd, mk(c.dx, c.dy, c.dz));
  if (fabs(cos_ray_cone) != 1.) {
    h.n = 1;
    h.s[0] = Seg{pin, pout};
  } else {
    h.n = 2;
    h.s[0] = cone_half_infinite(c, rd, pout);
    h.s[1] = cone_half_infinite(c, rd, pin);
  }
}

// ------------------------------------------------------------- cylinder
__device__ __forceinline__ void cylinder_hit(const JshModel& m, V3 ro_cm, V3 rd, Hits& h) {
  h.n = 0;
  V3 ro = vdiv(ro_cm, JSH_PC);
  V3 co = vdiv(mk(m.gox, m.goy, m.goz), JSH_PC);
  V3 cd = mk(m.gdx, m.gdy, m.gdz);
  V3 delta = vsub(ro, co);
  V3 v = vsub(rd, vmul(cd, vdot(rd, cd)));
  double c2 = vsq(v);
  V3 w = vsub(delta, vmul(cd, vdot(delta, cd)));
  double c1 = vdot(v, w);
  double c0 = sb(vsq(w), dv(m.r, JSH_PC));
  double d = sb(ml(c1, c1), ml(c0, c2));
  if (d < 0) return;
  if (d > 0) {
    double eps = (c1 > 0 ? 1 : -1);
    double s = sq(d);
    double den = sb(-c1, ml(eps, s));
    double t1 = dv(den, c2);
    double t2 = dv(c0, den);
    h.n = 1;
    h.s[0] = Seg{ray_point(ro_cm, rd, ml(JSH_PC, fmin(t1, t2))), ray_point(ro_cm, rd, ml(JSH_PC, fmax(t1, t2)))};
    return;
  }
  V3 go = mk(m.gox, m.goy, m.goz);
  if (c2 == 1 && c1 == 0 && c0 == 0) {
    V3 p = ray_point(ro_cm, rd, dv(-c1, c2));
    h.n = 1;
    h.s[0] = Seg{p, p};
  } else if (c2 == 0 && c1 == 0 && c0 == 0) {
    h.n = 1;
    h.s[0] = full_infinite(ro_cm, rd, go, ml(100., m.r));
  } else if (c2 == 0 && c1 == 0 && c0 > 0) {
    return;
  } else if (c2 == 0 && c1 == 0 && c0 <= 0) {
    h.n = 1;
    h.s[0] = full_infinite(ro_cm, rd, go, ml(100., m.r));
  } else {
    h.status |= JSH_ST_UB_GEOMETRY;
  }
}

// ------------------------------------------------------------ paraboloid
// General quadric roots (src/Geometry.cpp:28-69) for the paraboloid
// x^2 + y^2 + I z = 0 (A = B = 1, I = -r0^2/pc, the rest zero), keeping the
// reference's full left-to-right expression so zero terms round identically.
__device__ __forceinline__ int quadric_paraboloid(V3 R0, V3 Rd, double I, double ts[2]) {
  const double A = 1., B = 1., Cc = 0., D = 0., E = 0., F = 0., G = 0., H = 0., J = 0.;
  double x0 = R0.x, y0 = R0.y, z0 = R0.z;
  double xd = Rd.x, yd = Rd.y, zd = Rd.z;
  double Aq = ad(ad(ad(ad(ad(ml(ml(A, xd), xd), ml(ml(B, yd), yd)), ml(ml(Cc, zd), zd)), ml(ml(D, xd), yd)),
                    ml(ml(E, xd), zd)),
                 ml(ml(F, yd), zd));
  double Bq = ml(ml(ml(2., A), x0), xd);
  Bq = ad(Bq, ml(ml(ml(2., B), y0), yd));
  Bq = ad(Bq, ml(ml(ml(2., Cc), z0), zd));
  Bq = ad(Bq, ml(D, ad(ml(x0, yd), ml(y0, xd))));
  Bq = ad(Bq, ml(ml(E, x0), zd));
  Bq = ad(Bq, ml(F, ad(ml(y0, zd), ml(yd, z0))));
  Bq = ad(Bq, ml(G, xd));
  Bq = ad(Bq, ml(H, yd));
  Bq = ad(Bq, ml(I, zd));
  double Cq = ml(ml(A, x0), x0);
  Cq = ad(Cq, ml(ml(B, y0), y0));
  Cq = ad(Cq, ml(ml(Cc, z0), z0));
  Cq = ad(Cq, ml(ml(D, x0), y0));
  Cq = ad(Cq, ml(ml(E, x0), z0));
  Cq = ad(Cq, ml(ml(F, y0), z0));
  Cq = ad(Cq, ml(G, x0));
  Cq = ad(Cq, ml(H, y0));
  Cq = ad(Cq, ml(I, z0));
  Cq = ad(Cq, J);
  double Dscr = sb(ml(Bq, Bq), ml(ml(4., Aq), Cq));
  if (Aq == 0) {
    ts[0] = dv(-Cq, Bq);
    return 1;
  }
  if (Dscr < 0) return 0;
  double t0 = dv(sb(-Bq, sq(Dscr)), ml(2., Aq));
  if (t0 > 0) {
    ts[0] = t0;
    return 1;
  }
  ts[0] = t0;
  ts[1] = dv(ad(-Bq, sq(Dscr)), ml(2., Aq));
  return 2;
}

__device__ __forceinline__ void parabaloid_hit(double r0, V3 ro, V3 rd, Hits& h) {
  h.n = 0;
  double ts[2];
  int n = quadric_paraboloid(ro, rd, dv(ml(-r0, r0), JSH_PC), ts);
  if (n == 2) {
    h.n = 1;
    h.s[0] = Seg{ray_point(ro, rd, fmin(ts[0], ts[1])), ray_point(ro, rd, fmax(ts[0], ts[1]))};
  }
}

__device__ __forceinline__ void parabaloid_cone_hit(const JshModel& m, V3 ro, V3 rd, Hits& h) {
  Hits hc, hp;
  hc.status = 0;
  hp.status = 0;
  cone_hit(m.cone, ro, rd, hc);
  parabaloid_hit(m.r0, ro, rd, hp);
  h.n = 0;
  h.status |= hc.status | hp.status;
  if (hc.n == 0 && hp.n == 0) return;
  if (hc.n != 0 && hp.n == 0) {
    if (hc.s[0].in.z > m.z0) {
      h.n = hc.n;
      h.s[0] = hc.s[0];
      h.s[1] = hc.s[1];
    }
    return;
  }
  if (hc.n == 0) {
    h.status |= JSH_ST_UB_GEOMETRY;
    return;
  }
  V3 pin = (hp.s[0].in.z > m.z0) ? hc.s[0].in : hp.s[0].in;
  V3 pout = (hp.s[0].out.z < m.z0) ? hp.s[0].out : hc.s[0].out;
  h.n = 1;
  h.s[0] = Seg{pin, pout};
}

// ------------------------------------------------------- SimulationGeometry
// Line / revolved-hull intersection (src/Geometry.cpp:97-132: the LINE
// through the ray, in pc, against the convex hull of the revolved grid
// points; the two points scaled back to cm).  The hull is the intersection
// over the n_circle azimuthal sectors k of the slabs {g_k . (x, y) <= R(z),
// z_min <= z <= z_max} (see jsh_hull.cpp).  Along the line, with z as the
// parameter (d_z != 0), slab k is the z interval where
// D(z) = R(z) - (A + B z) >= 0, A + B z the line's g_k coordinate; D is
// concave and piecewise linear with breaks at the profile vertices, so its
// sign at the vertices (binary searches) finds the profile edge or the cap
// that the line crosses on each side, and the crossing parameter comes from
// that edge's half-plane.  The segment is [max_k t_in, min_k t_out].
// point_in is the point of smaller t (the reference orders CGAL's two
// points by the sign of x, which agrees when they straddle x = 0 and is
// the AABB traversal order otherwise).
__device__ __forceinline__ double hull_D(const JshHull& H, int i, double A, double B) {
  return sb(H.vR[i], ad(A, ml(B, H.vz[i])));
}
// t where the line crosses the half-plane of edge e (sector coordinates u0 +
// t u1 of the line); a line parallel to the edge (beta == 0, only through
// rounding) takes the t of the edge's lower vertex height.
__device__ __forceinline__ double hull_edge_t(const JshHull& H, int e, double u0, double u1, double oz, double dz) {
  const double a = H.abc[3 * e], b = H.abc[3 * e + 1], c = H.abc[3 * e + 2];
  const double alpha = sb(ad(ml(a, u0), ml(b, oz)), c);
  const double beta = ad(ml(a, u1), ml(b, dz));
  if (beta == 0.0) return dv(sb(H.vz[e], oz), dz);
  return dv(-alpha, beta);
}

static __device__ __noinline__ void simulation_hit(const JshHull& H, V3 ro_cm, V3 rd, Hits& h) {
  const V3 o = vdiv(ro_cm, JSH_PC);
  const int m = H.m;
  double tlo = -INFINITY, thi = INFINITY;
  if (rd.z == 0.0) {
    // the line stays at z = o.z: one radius bound R(o.z) for every sector
    if (!(o.z >= H.z_min && o.z <= H.z_max)) return;
    int lo = 0, hi = m;  // edge e with vz[e] <= o.z <= vz[e+1]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (H.vz[mid] <= o.z) lo = mid;
      else hi = mid;
    }
    const double a = H.abc[3 * lo], b = H.abc[3 * lo + 1], c = H.abc[3 * lo + 2];
    const double R0 = dv(sb(c, ml(b, o.z)), a);
    for (int k = 0; k < H.n_circle; ++k) {
      const double gx = H.g[2 * k], gy = H.g[2 * k + 1];
      const double u0 = ad(ml(gx, o.x), ml(gy, o.y)), u1 = ad(ml(gx, rd.x), ml(gy, rd.y));
      if (u1 > 0.0) thi = fmin(thi, dv(sb(R0, u0), u1));
      else if (u1 < 0.0) tlo = fmax(tlo, dv(sb(R0, u0), u1));
      else if (u0 > R0) return;
    }
  } else {
    const double t_zmin = dv(sb(H.z_min, o.z), rd.z), t_zmax = dv(sb(H.z_max, o.z), rd.z);
    for (int k = 0; k < H.n_circle; ++k) {
      const double gx = H.g[2 * k], gy = H.g[2 * k + 1];
      const double u0 = ad(ml(gx, o.x), ml(gy, o.y)), u1 = ad(ml(gx, rd.x), ml(gy, rd.y));
      const double B = dv(u1, rd.z), A = sb(u0, ml(B, o.z));
      // vertex of D's maximum: the first edge whose slope falls below B
      int lo = 0, hi = m;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (sb(sb(H.vR[mid + 1], H.vR[mid]), ml(B, sb(H.vz[mid + 1], H.vz[mid]))) < 0.0) hi = mid;
        else lo = mid + 1;
      }
      const int top = lo;
      if (!(hull_D(H, top, A, B) >= 0.0)) return;  // this sector's slab misses the line
      double ta, tb;
      if (hull_D(H, 0, A, B) >= 0.0) {
        ta = t_zmin;
      } else {
        int l = 0, r = top;  // D(l) < 0 <= D(r)
        while (r - l > 1) {
          const int mid = (l + r) >> 1;
          if (hull_D(H, mid, A, B) >= 0.0) r = mid;
          else l = mid;
        }
        ta = hull_edge_t(H, l, u0, u1, o.z, rd.z);
      }
      if (hull_D(H, m, A, B) >= 0.0) {
        tb = t_zmax;
      } else {
        int l = top, r = m;  // D(l) >= 0 > D(r)
        while (r - l > 1) {
          const int mid = (l + r) >> 1;
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
    // tangent (one point): the reference reads a second point that CGAL did
    // not return
    if (tlo == thi) h.status |= JSH_ST_UB_GEOMETRY;
    return;
  }
  h.n = 1;
  h.s[0].in = vmul(ray_point(o, rd, tlo), JSH_PC);
  h.s[0].out = vmul(ray_point(o, rd, thi), JSH_PC);
}

__device__ __forceinline__ void geo_hit(const JshModel& m, V3 ro, V3 rd, Hits& h) {
  h.n = 0;
  h.status = 0;
  switch (m.geo_kind) {
    case JSH_GEO_CONE: cone_hit(m.cone, ro, rd, h); break;
    case JSH_GEO_CYLINDER: cylinder_hit(m, ro, rd, h); break;
    case JSH_GEO_PARABALOID: parabaloid_hit(m.r0, ro, rd, h); break;
    case JSH_GEO_PARABALOID_CONE: parabaloid_cone_hit(m, ro, rd, h); break;
    case JSH_GEO_SIMULATION: simulation_hit(m.hull, ro, rd, h); break;
    default: break;
  }
}

}  // namespace jsh
