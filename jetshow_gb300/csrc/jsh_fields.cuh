// jsh_fields.cuh -- FP64 field laws, Lorentz kinematics and synchrotron
// transfer coefficients on the device, written as the reference writes them
// (src/VField.cpp:25-274, src/BField.cpp:35-224, src/NField.cpp:5-60,
// src/utils.cpp:8-173, src/Jet.cpp:15-46, :218-237), plus the gridded-field
// lookup (src/SimulationInterpolater.cpp:43-102) on a uniform bucket grid.
// This is the all-FP64 "plain" form; the mixed-precision form lives in
// jsh_fields_mixed.cuh.
#pragma once

#include "jsh_geometry.cuh"
#include "jsh_random.h"

namespace jsh {

// Plain (contractible) vector helpers for the transfer math.
struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 d3(double x, double y, double z) { return D3{x, y, z}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D3 operator*(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ D3 operator/(D3 a, double s) { return d3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ double dot(D3 a, D3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ double norm(D3 a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ D3 cross(D3 a, D3 b) {
  return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// ---------------------------------------------------------- gridded field
// Containing triangle of (px, py) = (z, r) [pc] by the bucket list, then
// barycentric weights; nan_value outside the hull or on NaN.  Every
// operation is an explicitly rounded FP64 intrinsic in a fixed order (no
// contraction into fma), the order the oracle's plain-C restatement rounds
// in: the orientation determinants (b - a) x (c - a) as
// (bx - ax)(cy - ay) - (by - ay)(cx - ax), each weight one division by the
// triangle's, the value ((w0 v0 + w1 v1) + w2 v2).  With that, the device
// and the oracle accept the same first triangle of a bucket's ascending list
// and return the same bits.
__device__ __forceinline__ double orient2_rn(double ax, double ay, double bx, double by, double cx, double cy) {
  return __dsub_rn(__dmul_rn(__dsub_rn(bx, ax), __dsub_rn(cy, ay)), __dmul_rn(__dsub_rn(by, ay), __dsub_rn(cx, ax)));
}

__device__ inline double grid_value(const JshGrid& G, int field, double px, double py, double nan_value) {
  if (G.n_tri == 0) return nan_value;
  if (!(px >= G.x0 && py >= G.y0)) return nan_value;
  int i = (int)floor(__ddiv_rn(__dsub_rn(px, G.x0), G.h)), j = (int)floor(__ddiv_rn(__dsub_rn(py, G.y0), G.h));
  if (i >= G.nbx) i = G.nbx - 1;
  if (j >= G.nby) j = G.nby - 1;
  if (i < 0 || j < 0) return nan_value;
  int b = j * G.nbx + i;
  int q0 = G.bstart[b], q1 = G.bstart[b + 1];
  for (int q = q0; q < q1; ++q) {
    int t = G.bitems[q];
    int v0 = G.tri[3 * t], v1 = G.tri[3 * t + 1], v2 = G.tri[3 * t + 2];
    double ax = G.xy[2 * v0], ay = G.xy[2 * v0 + 1];
    double bx = G.xy[2 * v1], by = G.xy[2 * v1 + 1];
    double cx = G.xy[2 * v2], cy = G.xy[2 * v2 + 1];
    double area = orient2_rn(ax, ay, bx, by, cx, cy);
    if (area == 0) continue;
    double w0 = __ddiv_rn(orient2_rn(px, py, bx, by, cx, cy), area);
    double w1 = __ddiv_rn(orient2_rn(ax, ay, px, py, cx, cy), area);
    double w2 = __ddiv_rn(orient2_rn(ax, ay, bx, by, px, py), area);
    if (w0 < 0 || w1 < 0 || w2 < 0) continue;
    double val = __dadd_rn(__dadd_rn(__dmul_rn(w0, (double)G.val[(int64_t)v0 * G.n_fields + field]),
                                     __dmul_rn(w1, (double)G.val[(int64_t)v1 * G.n_fields + field])),
                           __dmul_rn(w2, (double)G.val[(int64_t)v2 * G.n_fields + field]));
    if (isnan(val)) return nan_value;
    return val;
  }
  return nan_value;
}

// (x, y, z) [cm] -> (z/pc, hypot(x, y)/pc) (src/SimulationInterpolater.cpp:46-50),
// the cylindrical radius as sqrt(x^2 + y^2) in correctly rounded steps
// (within an ulp of a libm hypot for these magnitudes; the oracle rounds
// the same way).
__device__ __forceinline__ double sim_value(const JshGrid& G, int field, D3 p, double nan_value) {
  double x = __ddiv_rn(p.x, JSH_PC), y = __ddiv_rn(p.y, JSH_PC), z = __ddiv_rn(p.z, JSH_PC);
  return grid_value(G, field, z, __dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y))), nan_value);
}

// ---------------------------------------------------------------- V
__device__ __forceinline__ D3 v_central(double g, D3 o, D3 p) {
  double r = norm(p + o);
  double v_r = JSH_C * sqrt(1. - 1. / (g * g));
  return d3(v_r * (p.x + o.x) / r, v_r * (p.y + o.y) / r, v_r * (p.z + o.z) / r);
}
__device__ __forceinline__ D3 v_sheared_central(double ga, double gb, double th, D3 o, D3 p) {
  double r = norm(p + o);
  double theta = acos(p.z + o.z / r);
  double g = ga - (ga - gb) * theta / th;
  double v_r = JSH_C * sqrt(1. - 1. / (g * g));
  return d3(v_r * (p.x + o.x) / r, v_r * (p.y + o.y) / r, v_r * (p.z + o.z) / r);
}
__device__ __forceinline__ D3 v_parabolic_dir(double v_r, double Rz0, D3 p) {
  double r = hypot(p.x, p.y);
  double R = sqrt(Rz0 * Rz0 * p.z / JSH_PC);
  double r0 = Rz0 * r / R;
  double alpha = atan(2 * JSH_PC * r / r0 / r0);
  if (r == 0) return d3(0, 0, v_r);
  return d3(v_r * cos(alpha) * p.x / r, v_r * cos(alpha) * p.y / r, v_r * sin(alpha));
}
__device__ __forceinline__ D3 v_acc_parabolic(double g0, double R0, double Rz0, D3 p) {
  double gamma = 1 + (g0 - 1) / sqrt(R0) * sqrt(p.z);
  return v_parabolic_dir(JSH_C * sqrt(1. - 1. / (gamma * gamma)), Rz0, p);
}
__device__ __forceinline__ D3 v_sheared_acc_parabolic(double ga0, double gb0, double R0, double Rz0, D3 p) {
  double r = hypot(p.x, p.y);
  double R0_border = sqrt(Rz0 * Rz0 * R0 / JSH_PC);
  double R = sqrt(Rz0 * Rz0 * p.z / JSH_PC);
  double rR0 = R0_border * r / R;
  double gamma0 = ga0 - (ga0 - gb0) * pow(rR0 / R0_border, 0.25);
  if (gamma0 < 1) gamma0 = 1;
  double gamma = 1 + (gamma0 - 1) / sqrt(R0) * sqrt(p.z);
  return v_parabolic_dir(JSH_C * sqrt(1. - 1. / (gamma * gamma)), Rz0, p);
}

__device__ inline D3 vfield(const JshModel& m, D3 p) {
  const double* q = m.vp;
  switch (m.v_kind) {
    case JSH_V_CONST_FLAT: return d3(0, 0, JSH_C * sqrt(1. - 1. / (q[0] * q[0])));
    case JSH_V_SHEARED_FLAT: {
      double r = sqrt(p.x * p.x + p.y * p.y);
      double g = q[0] - (q[0] - q[1]) * r / q[2];
      return d3(0, 0, JSH_C * sqrt(1. - 1. / (g * g)));
    }
    case JSH_V_SHEATH_FLAT: {
      double r = sqrt(p.x * p.x + p.y * p.y);
      double g = (r < q[2]) ? q[0] : q[1];
      return d3(0, 0, JSH_C * sqrt(1. - 1. / (g * g)));
    }
    case JSH_V_CONST_CENTRAL: return v_central(q[0], d3(q[1], q[2], q[3]), p);
    case JSH_V_SHEARED_CENTRAL: return v_sheared_central(q[0], q[1], q[2], d3(q[3], q[4], q[5]), p);
    case JSH_V_SHEATH_CENTRAL: {
      D3 o = d3(q[3], q[4], q[5]);
      double r = norm(p + o);
      double theta = acos(p.z / r);
      double g = (theta < q[2]) ? q[0] : q[1];
      double v_r = JSH_C * sqrt(1. - 1. / (g * g));
      return d3(v_r * (p.x + o.x) / r, v_r * (p.y + o.y) / r, v_r * (p.z + o.z) / r);
    }
    case JSH_V_CONST_PARABOLIC: return v_parabolic_dir(JSH_C * sqrt(1. - 1. / (q[0] * q[0])), q[1], p);
    case JSH_V_ACC_PARABOLIC: return v_acc_parabolic(q[0], q[1], q[2], p);
    case JSH_V_SHEARED_ACC_PARABOLIC: return v_sheared_acc_parabolic(q[0], q[1], q[2], q[3], p);
    case JSH_V_ACC_PARABOLIC_CONST_CONE:
      if (p.z > q[2]) return v_central(q[0], d3(0, 0, m.v_cone_oz), p);
      return v_acc_parabolic(q[0], q[2], q[1], p);
    case JSH_V_SHEARED_ACC_PARABOLIC_CONST_CONE:
      if (p.z > q[3]) return v_sheared_central(q[0], q[1], m.v_theta, d3(0, 0, m.v_cone_oz), p);
      return v_sheared_acc_parabolic(q[0], q[1], q[3], q[2], p);
    case JSH_V_SIMULATION: {
      double g = sim_value(m.grids[2], m.f_v, p, 1.0);
      return d3(0, 0, JSH_C * sqrt(1. - 1. / (g * g)));
    }
    default: return d3(0, 0, 0);
  }
}

// ---------------------------------------------------------------- B
__device__ inline double bscalar(const JshModel& m, D3 p) {
  const double* q = m.bp;
  switch (m.b_kind) {
    case JSH_B_RANDOM_SCALAR: return q[0] * pow(norm(p) / JSH_PC, -q[1]);
    case JSH_B_RANDOM_SCALAR_Z: return q[0] * pow(fabs(p.z) / JSH_PC, -q[1]);
    case JSH_B_COMPOSITE_RANDOM_SCALAR_Z: {
      double r = fabs(p.z);
      if (r > q[3]) return q[0] * pow(fabs(p.z) / JSH_PC, -q[2]);
      return q[0] * pow(fabs(p.z) / JSH_PC, -q[1]);
    }
    default: return 0.0;
  }
}

__device__ inline D3 bvector(const JshModel& m, D3 p) {
  const double* q = m.bp;
  switch (m.b_kind) {
    case JSH_B_CONST_CYLINDER: return d3(0.0, 0.0, q[0] * pow(norm(p) / JSH_PC, -q[1]));
    case JSH_B_CONST_CYLINDER_Z: return d3(0.0, 0.0, q[0] * pow(fabs(p.z) / JSH_PC, -q[1]));
    case JSH_B_RADIAL_CONICAL: {
      double r = norm(p);
      double b = q[0] * pow(r / JSH_PC, -q[1]);
      return d3(b * p.x / r, b * p.y / r, b * p.z / r);
    }
    case JSH_B_TOROIDAL: {
      double fi = atan(p.y / p.x);
      double b = q[0] * pow(p.z / JSH_PC, -q[1]);
      return d3(-sin(fi) * b, cos(fi) * b, 0);
    }
    case JSH_B_HELICAL_CYLINDER: {
      double r = sqrt(p.x * p.x + p.y * p.y);
      return d3(q[0] * tan(q[1] * p.y / r), -q[0] * tan(q[1] * p.x / r), q[0]);
    }
    case JSH_B_SPIRAL_CONICAL: {
      double b_z = q[0] / (p.z * p.z / (JSH_PC * JSH_PC));
      return d3(b_z * (p.x / p.z + p.y * m.tan_pitch / JSH_PC), b_z * (p.y / p.z - p.x * m.tan_pitch / JSH_PC), b_z);
    }
    case JSH_B_FORCE_FREE_CYLINDRICAL: {
      double fi = atan(p.y / p.x);
      return d3(-q[0] * m.bessel1 * sin(fi), q[0] * m.bessel1 * sin(fi), q[0] * m.bessel0);
    }
    case JSH_B_HELICAL_CONICAL: {
      double b = q[0] * pow(norm(p) / JSH_PC, -q[1]);
      double rc = sqrt(p.x * p.x + p.y * p.y);
      double px = 0.0, py = 0.0;
      if (rc > 0.0) {
        px = -p.y / rc;
        py = p.x / rc;
        if (q[3] != 0.0 && p.x < 0.0) {
          px = -px;
          py = -py;
        }
      }
      double bt = b * m.sin_pitch;
      return d3(bt * px, bt * py, b * m.cos_pitch);
    }
    case JSH_B_SIMULATION: {
      double fi = atan(p.y / p.x);
      double bp = sim_value(m.grids[0], m.fb_p, p, 0.0);
      double bphi = sim_value(m.grids[0], m.fb_phi, p, 0.0);
      return d3(-sin(fi) * bphi, cos(fi) * bphi, bp);
    }
    default: return d3(0, 0, 0);
  }
}

// ---------------------------------------------------------------- N
__device__ inline double nfield(const JshModel& m, D3 p) {
  const double* q = m.np;
  switch (m.n_kind) {
    case JSH_N_CONST: return q[0];
    case JSH_N_BK: return q[0] * pow(norm(p) / JSH_PC, -q[1]);
    case JSH_N_BKZ: return q[0] * pow(fabs(p.z) / JSH_PC, -q[1]);
    case JSH_N_COMPOSITE_BK: {
      double z = fabs(p.z);
      if (z > q[3]) return q[0] * pow(norm(p) / JSH_PC, -q[2]);
      return q[0] * pow(norm(p) / JSH_PC, -q[1]);
    }
    case JSH_N_SIMULATION: return sim_value(m.grids[1], m.f_n, p, 0.0);
    default: return 0.0;
  }
}

// ------------------------------------------------------- random directions
// The cell nearest to p [cm] (RandomCells::getID, src/Cells.cpp:13-18: the
// smallest squared distance, the lowest index among equals), the squared
// distances rounded in a fixed order; p's bucket lists every cell that can
// be nearest inside it, a point outside the grid scans every cell.
__device__ inline int cells_nearest64(const JshCells& C, D3 p) {
  const double fx = __ddiv_rn(__dsub_rn(p.x, C.x0), C.h), fy = __ddiv_rn(__dsub_rn(p.y, C.y0), C.h),
               fz = __ddiv_rn(__dsub_rn(p.z, C.z0), C.h);
  const bool inside = fx >= 0.0 && fy >= 0.0 && fz >= 0.0 && fx < (double)C.nbx && fy < (double)C.nby &&
                      fz < (double)C.nbz;
  int q0 = 0, q1 = C.n;
  const int32_t* list = nullptr;
  if (inside) {
    const int b = ((int)fz * C.nby + (int)fy) * C.nbx + (int)fx;
    q0 = C.bstart[b];
    q1 = C.bstart[b + 1];
    list = C.bitems;
  }
  double best = INFINITY;
  int bi = 0;
  for (int q = q0; q < q1; ++q) {
    const int c = list ? list[q] : q;
    const double dx = __dsub_rn(p.x, C.p[3 * c]), dy = __dsub_rn(p.y, C.p[3 * c + 1]),
                 dz = __dsub_rn(p.z, C.p[3 * c + 2]);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (d2 < best) {
      best = d2;
      bi = c;
    }
  }
  return bi;
}

// RandomVectorBField::bf (src/BField.cpp:154-161): b + fraction |b| n, n the
// nearest cell's direction or a fresh counter-based draw keyed by (pixel,
// frequency, evaluation index).
__device__ inline D3 brandom64(const JshModel& m, D3 b, D3 p, uint32_t k0, uint32_t k1, uint32_t k2) {
  double n[3];
  if (m.rnd_kind == JSH_RND_CELLS) {
    const int c = cells_nearest64(m.cells, p);
    n[0] = m.cells.dir[3 * c];
    n[1] = m.cells.dir[3 * c + 1];
    n[2] = m.cells.dir[3 * c + 2];
  } else {
    jsh_random_direction(m.rnd_seed, k0, k1, k2, n);
  }
  const double f = m.rnd_frac * norm(b);
  return d3(b.x + f * n[0], b.y + f * n[1], b.z + f * n[2]);
}

// ------------------------------------------------------- coefficients
enum { CK_I = 0, CK_Q, CK_V, CK_F, CK_C, CE_I, CE_Q, CE_V, NCOEF };

// Lab-frame coefficients at p for LOS n_los (towards the observer):
// k = k'/D and eta = eta' D D with k', eta' evaluated on the plasma-frame
// B', n', nu' = nu/D and n_los'.  kU = etaU = hQ = 0 (src/utils.cpp:67-69,
// :101-103, :136-138) and are not stored.  FULL = false computes kI, etaI.
// (rk0, rk1, rk2): key of a per-evaluation random direction (pixel,
// frequency, evaluation index), used by JSH_RND_POINTS only.
template <bool FULL>
__device__ inline void coefficients64(const JshModel& m, D3 p, D3 nl, double nu, double* k, uint32_t rk0 = 0,
                                      uint32_t rk1 = 0, uint32_t rk2 = 0) {
  D3 v = vfield(m, p);
  D3 beta = v / JSH_C;
  double gamma = sqrt(1. / (1. - dot(beta, beta)));
  double D = 1. / (gamma * (1. - dot(beta, nl)));
  double n = nfield(m, p);
  double n_prime = m.n_plasma ? n : n / gamma;
  double nu_prime = nu / D;
  double s = m.s;
  double np = sqrt(n_prime * JSH_Q_E * JSH_Q_E / (JSH_PI * JSH_M_E));
  if (m.b_scalar) {
    double b = bscalar(m, p);
    double nb = JSH_Q_E * b / (2. * JSH_PI * JSH_M_E * JSH_C);
    double k0 = JSH_PI * np * np * nb / (JSH_C * nu_prime * nu_prime);
    double ki = k0 * pow(nb / nu_prime, s / 2.) * (m.fk_i * m.rnd_k);
    double e0 = JSH_PI * np * np * nb * JSH_M_E / JSH_C;
    double ei = e0 * pow(nb / nu_prime, (s - 1.) / 2.) * (m.fe_i * m.rnd_e);
    k[CK_I] = ki / D;
    k[CE_I] = ei * D * D;
    if (FULL) {
      k[CK_Q] = k[CK_V] = k[CK_F] = k[CK_C] = 0.0;
      k[CE_Q] = k[CE_V] = 0.0;
    }
    return;
  }
  D3 bl = bvector(m, p);
  if (m.rnd_kind != JSH_RND_NONE) bl = brandom64(m, bl, p, rk0, rk1, rk2);
  D3 b;
  if (m.b_plasma) {
    b = bl;
  } else {
    double s1 = gamma / ((1. + gamma) * (JSH_C * JSH_C));
    double vb = dot(v, bl);
    b = bl / gamma + d3(s1 * v.x * vb, s1 * v.y * vb, s1 * v.z * vb);
  }
  double df = D;
  D3 nlp = nl * df - beta * ((df + 1.) * (gamma / (gamma + 1.)));
  double nb = JSH_Q_E * norm(cross(nlp, b)) / (2. * JSH_PI * JSH_M_E * JSH_C);
  double k0 = JSH_PI * np * np * nb / (JSH_C * nu_prime * nu_prime);
  double ki = k0 * pow(nb / nu_prime, s / 2.) * m.fk_i;
  double e0 = JSH_PI * np * np * nb * JSH_M_E / JSH_C;
  double ei = e0 * pow(nb / nu_prime, (s - 1.) / 2.) * m.fe_i;
  k[CK_I] = ki / D;
  k[CE_I] = ei * D * D;
  if (!FULL) return;
  double bn = norm(b);
  double cos_theta = dot(b, nlp) / bn;
  double nbv = JSH_Q_E * bn / (2. * JSH_PI * JSH_M_E * JSH_C);
  double k0v = JSH_PI * np * np * nbv / (JSH_C * nu_prime * nu_prime);
  double kv = -k0v * cos_theta * pow(nb / nu_prime, (s + 1.) / 2.) * m.fk_v;
  double kfc = 2. * JSH_PI * np * np * nbv * cos_theta / (JSH_C * nu_prime * nu_prime);
  double kcc = -JSH_PI * np * np * nb * nb / (JSH_C * nu_prime * nu_prime * nu_prime);
  double kf = m.kfr_factor * kfc;
  double kc = m.kcr_a * (m.kcr_b - pow(nb / nu_prime, (s - 2.) / 2.)) * kcc;
  if (m.thermal_fraction != 0.0) {
    double npt = sqrt(m.thermal_fraction * n_prime * JSH_Q_E * JSH_Q_E / (JSH_PI * JSH_M_E));
    kf = kf + 2. * JSH_PI * npt * npt * nbv * cos_theta / (JSH_C * nu_prime * nu_prime);
    kc = kc + -JSH_PI * npt * npt * nb * nb / (JSH_C * nu_prime * nu_prime * nu_prime);
  }
  double e0v = JSH_PI * np * np * nbv * JSH_M_E / JSH_C;
  double ev = -e0v * cos_theta * pow(nb / nu_prime, s / 2.) * m.fe_v;
  k[CK_Q] = (m.kq_ratio * ki) / D;
  k[CK_V] = kv / D;
  k[CK_F] = kf / D;
  k[CK_C] = kc / D;
  k[CE_Q] = (m.eq_ratio * ei) * D * D;
  k[CE_V] = ev * D * D;
}

}  // namespace jsh
