// jsh_fields32.cuh -- FP32 field laws and transfer coefficients of the
// mixed-precision path.  Lengths are in pc, intensities in units of the
// per-frequency scale S (JshFreqConst::scale).
//
// Coefficient algebra.  With b = |n'_los x B'| (B', n' in the plasma frame),
// w = b D, P = w^((s+2)/2) and R = w^((s+1)/2) = P / sqrt(w), the lab-frame
// coefficients of src/utils.cpp:39-143 with k = k'/D and eta = eta' D^2
// (src/Jet.cpp:15-46, :218-237) collapse to
//   k_I   = a_k  n' P                      eta_I = a_e n' R D
//   k_Q   = q_k k_I                        eta_Q = q_e eta_I
//   k_V   = -a_v n' B_par R D              eta_V = -a_ev n' B_par D^2 P / w
//   k_F   =  a_f n' B_par D                k_C   = -a_c n' (c1 w^2 - c2 P)
// (B_par = B'.n'_los), where the a_* hold every frequency-dependent power,
// the tgamma factors, the cgs constants and the unit scales; they are
// computed once per frequency on the host in FP64.  One log2, one exp2 and
// one rsqrt per evaluation replace the reference's pow and tgamma calls.
// Velocities are carried as (Gamma, unit direction) so that
// 1 - beta.n = (1 - beta) + beta |v_hat - n|^2 / 2 with
// 1 - beta = 1 / (Gamma^2 (1 + beta)) stays accurate in FP32.
#pragma once

#include "jsh_random.h"
#include "jsh_request.h"

namespace jsh {

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float fdot(F3 a, F3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ F3 fcross(F3 a, F3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// x^e for x > 0 by exp2(e log2 x); NaN for x < 0 like pow with a
// non-integer exponent, 0 -> +inf / 0 as pow.
__device__ __forceinline__ float fpow(float x, float e) { return exp2f(e * __log2f(x)); }

// Point location on a gridded field in FP32: the containing triangle of
// (z, r) [pc] among the few of its bucket, with barycentric weights (a point
// within 1e-6 of an edge is accepted by either neighbour: the interpolant is
// continuous there).  ok = false outside the hull.
struct GridW {
  int v0, v1, v2;
  float w0, w1, w2;
  bool ok;
};
// Barycentric weights of (px, py) in triangle t; true when inside (the
// -1e-6 tolerance of the bucket search).
__device__ __forceinline__ bool grid_tri32(const JshGrid& G, int t, float px, float py, GridW& g) {
  const int v0 = G.tri[3 * t], v1 = G.tri[3 * t + 1], v2 = G.tri[3 * t + 2];
  const float2 a = *reinterpret_cast<const float2*>(G.xyf + 2 * v0);
  const float2 bb = *reinterpret_cast<const float2*>(G.xyf + 2 * v1);
  const float2 c = *reinterpret_cast<const float2*>(G.xyf + 2 * v2);
  const float area = (bb.x - a.x) * (c.y - a.y) - (bb.y - a.y) * (c.x - a.x);
  if (area == 0.f) return false;
  const float ia = 1.f / area;
  const float w0 = ((bb.x - px) * (c.y - py) - (bb.y - py) * (c.x - px)) * ia;
  const float w1 = ((px - a.x) * (c.y - a.y) - (py - a.y) * (c.x - a.x)) * ia;
  const float w2 = 1.f - w0 - w1;
  if (w0 >= -1e-6f && w1 >= -1e-6f && w2 >= -1e-6f) {
    g = GridW{v0, v1, v2, w0, w1, w2, true};
    return true;
  }
  return false;
}

// Point location of (px, py).  `hint` (may be null): the triangle of the
// lane's previous evaluation, tried first -- consecutive evaluation points
// along a ray mostly fall in the same triangle, and the bucket search costs
// a chain of dependent loads per candidate (bucket, list, triangle,
// vertices); the found triangle is stored back.  The hint restarts with
// each item, so an item's lookups do not depend on the lane that runs it.
__device__ inline GridW grid_locate32(const JshGrid& G, float px, float py, int* hint = nullptr) {
  GridW g;
  g.ok = false;
  if (G.n_tri == 0) return g;
  if (hint && *hint >= 0 && grid_tri32(G, *hint, px, py, g)) return g;
  const float fx = (px - G.x0f) * G.inv_hf, fy = (py - G.y0f) * G.inv_hf;
  if (!(fx >= 0.f && fy >= 0.f)) return g;
  const int i = min((int)fx, G.nbx - 1), j = min((int)fy, G.nby - 1);
  const int b = j * G.nbx + i;
  const int q1 = G.bstart[b + 1];
  for (int q = G.bstart[b]; q < q1; ++q) {
    const int t = G.bitems[q];
    if (grid_tri32(G, t, px, py, g)) {
      if (hint) *hint = t;
      return g;
    }
  }
  return g;
}
__device__ __forceinline__ float grid_val32(const JshGrid& G, const GridW& g, int field, float nan_value) {
  if (!g.ok) return nan_value;
  const int64_t nf = G.n_fields;
  const float v = g.w0 * G.val[g.v0 * nf + field] + g.w1 * G.val[g.v1 * nf + field] +
                  g.w2 * G.val[g.v2 * nf + field];
  return isnan(v) ? nan_value : v;
}
// (z, r) in pc: one field of a gridded field
__device__ inline float sim32(const JshGrid& G, int field, F3 p, float nan_value) {
  return grid_val32(G, grid_locate32(G, p.z, sqrtf(p.x * p.x + p.y * p.y)), field, nan_value);
}

// ---------------------------------------------------------------- V
struct Vel {
  float gamma;
  F3 dir;  // unit
};

__device__ __forceinline__ F3 parabolic_dir(float Rz0_pc, F3 p) {
  float r = hypotf(p.x, p.y);
  if (r == 0.f) return f3(0.f, 0.f, 1.f);
  float R = sqrtf(Rz0_pc * Rz0_pc * p.z);
  float r0 = Rz0_pc * r / R;
  float alpha = atanf(2.f * r / r0 / r0);
  float sa, ca;
  sincosf(alpha, &sa, &ca);
  return f3(ca * p.x / r, ca * p.y / r, sa);
}

__device__ inline Vel vfield32(const JshModel& m, const JshMixed& X, F3 p) {
  const float* q = X.vq;
  const float* qp = X.vq_pc;
  const float inv_pc = (float)(1.0 / JSH_PC);
  switch (m.v_kind) {
    case JSH_V_CONST_FLAT: return Vel{q[0], f3(0, 0, 1)};
    case JSH_V_SHEARED_FLAT: {
      float r = sqrtf(p.x * p.x + p.y * p.y);
      float g = q[0] - X.v_dq01 * r / qp[2];
      return Vel{g, f3(0, 0, 1)};
    }
    case JSH_V_SHEATH_FLAT: {
      float r = sqrtf(p.x * p.x + p.y * p.y);
      return Vel{r < qp[2] ? q[0] : q[1], f3(0, 0, 1)};
    }
    case JSH_V_CONST_CENTRAL: {
      F3 a = p + f3(q[1], q[2], q[3]) * inv_pc;
      return Vel{q[0], a * rsqrtf(fdot(a, a))};
    }
    case JSH_V_SHEARED_CENTRAL: {
      // theta = acos(z + o_z / r) evaluated in cm as written (src/VField.cpp:83)
      F3 a = p + f3(q[3], q[4], q[5]) * inv_pc;
      float r_cm = sqrtf(fdot(a, a)) * (float)JSH_PC;
      float theta = acosf(p.z * (float)JSH_PC + q[5] / r_cm);
      float g = q[0] - X.v_dq01 * theta / q[2];
      return Vel{g, a * rsqrtf(fdot(a, a))};
    }
    case JSH_V_SHEATH_CENTRAL: {
      // theta = acos(z / |p + o|) < theta_sheath (src/VField.cpp): near a
      // small sheath angle acos in FP32 is ill-conditioned (1 - cos theta
      // ~ 2e-4 at 0.02 rad magnifies the rounding of z / r by 1/theta^2), so
      // for z > 0 the test compares 1 - cos theta = (|a|^2 - z^2) / (r (r + z)),
      // a = p + o, formed without cancellation, with 1 - cos theta_sheath
      F3 a = p + f3(q[3], q[4], q[5]) * inv_pc;
      float r = sqrtf(fdot(a, a));
      bool spine;
      if (p.z > 0.f) {
        const float oz = q[5] * inv_pc;
        const float num = fmaf(a.x, a.x, fmaf(a.y, a.y, oz * (2.f * p.z + oz)));
        spine = num / (r * (r + p.z)) < X.v_omc;
      } else {
        spine = acosf(p.z / r) < q[2];
      }
      return Vel{spine ? q[0] : q[1], a * (1.f / r)};
    }
    case JSH_V_CONST_PARABOLIC: return Vel{q[0], parabolic_dir(qp[1], p)};
    case JSH_V_ACC_PARABOLIC: {
      float g = 1.f + X.v_g0m1 * sqrtf(p.z / qp[1]);
      return Vel{g, parabolic_dir(qp[2], p)};
    }
    case JSH_V_SHEARED_ACC_PARABOLIC:
    case JSH_V_SHEARED_ACC_PARABOLIC_CONST_CONE:
    case JSH_V_ACC_PARABOLIC_CONST_CONE: {
      int k = m.v_kind;
      float z0_pc = (k == JSH_V_ACC_PARABOLIC_CONST_CONE ? qp[2] : qp[3]);
      if (k != JSH_V_SHEARED_ACC_PARABOLIC && p.z > z0_pc) {
        F3 a = p + f3(0.f, 0.f, X.v_cone_oz_pc);
        F3 dir = a * rsqrtf(fdot(a, a));
        if (k == JSH_V_ACC_PARABOLIC_CONST_CONE) return Vel{q[0], dir};
        float r_cm = sqrtf(fdot(a, a)) * (float)JSH_PC;
        float theta = acosf(p.z * (float)JSH_PC + X.v_cone_oz / r_cm);
        return Vel{q[0] - X.v_dq01 * theta / X.v_theta, dir};
      }
      if (k == JSH_V_ACC_PARABOLIC_CONST_CONE) {
        float g = 1.f + X.v_g0m1 * sqrtf(p.z / z0_pc);
        return Vel{g, parabolic_dir(qp[1], p)};
      }
      float R0_pc = (k == JSH_V_SHEARED_ACC_PARABOLIC) ? qp[2] : z0_pc;
      float Rz0_pc = (k == JSH_V_SHEARED_ACC_PARABOLIC ? qp[3] : qp[2]);
      float r = hypotf(p.x, p.y);
      float R = sqrtf(Rz0_pc * Rz0_pc * p.z);
      float g0 = q[0] - X.v_dq01 * sqrtf(sqrtf(r / R));
      if (g0 < 1.f) g0 = 1.f;
      float g = 1.f + (g0 - 1.f) * sqrtf(p.z / R0_pc);
      return Vel{g, parabolic_dir(Rz0_pc, p)};
    }
    case JSH_V_SIMULATION: return Vel{sim32(m.grids[2], m.f_v, p, 1.0f), f3(0, 0, 1)};
    default: return Vel{1.f, f3(0, 0, 1)};
  }
}

// ---------------------------------------------------------------- N
__device__ inline float nfield32(const JshModel& m, const JshMixed& X, F3 p) {
  const float* q = X.nq;
  const float* qp = X.nq_pc;
  switch (m.n_kind) {
    case JSH_N_CONST: return q[0];
    case JSH_N_BK: return q[0] * fpow(sqrtf(fdot(p, p)), -q[1]);
    case JSH_N_BKZ: return q[0] * fpow(fabsf(p.z), -q[1]);
    case JSH_N_COMPOSITE_BK: {
      float e = (fabsf(p.z) > qp[3]) ? q[2] : q[1];
      return q[0] * fpow(sqrtf(fdot(p, p)), -e);
    }
    case JSH_N_SIMULATION: return sim32(m.grids[1], m.f_n, p, 0.0f);
    default: return 0.f;
  }
}

// ---------------------------------------------------------------- B
__device__ inline float bscalar32(const JshModel& m, const JshMixed& X, F3 p) {
  const float* q = X.bq;
  const float* qp = X.bq_pc;
  switch (m.b_kind) {
    case JSH_B_RANDOM_SCALAR: return q[0] * fpow(sqrtf(fdot(p, p)), -q[1]);
    case JSH_B_RANDOM_SCALAR_Z: return q[0] * fpow(fabsf(p.z), -q[1]);
    case JSH_B_COMPOSITE_RANDOM_SCALAR_Z: {
      float e = (fabsf(p.z) > qp[3]) ? q[2] : q[1];
      return q[0] * fpow(fabsf(p.z), -e);
    }
    default: return 0.f;
  }
}

// sin and cos of atan(u): u / sqrt(1 + u^2), 1 / sqrt(1 + u^2)
__device__ __forceinline__ void sincos_atan(float u, float& s, float& c) {
  if (isinf(u)) {
    s = u > 0 ? 1.f : -1.f;
    c = 0.f;
    return;
  }
  c = rsqrtf(fmaf(u, u, 1.f));
  s = u * c;
}

__device__ inline F3 bvector32(const JshModel& m, const JshMixed& X, F3 p) {
  const float* q = X.bq;
  switch (m.b_kind) {
    case JSH_B_CONST_CYLINDER: return f3(0, 0, q[0] * fpow(sqrtf(fdot(p, p)), -q[1]));
    case JSH_B_CONST_CYLINDER_Z: return f3(0, 0, q[0] * fpow(fabsf(p.z), -q[1]));
    case JSH_B_RADIAL_CONICAL: {
      float r = sqrtf(fdot(p, p));
      return p * (q[0] * fpow(r, -q[1]) / r);
    }
    case JSH_B_TOROIDAL: {
      float s, c;
      sincos_atan(p.y / p.x, s, c);
      float b = q[0] * fpow(p.z, -q[1]);
      return f3(-s * b, c * b, 0.f);
    }
    case JSH_B_HELICAL_CYLINDER: {
      float r = sqrtf(p.x * p.x + p.y * p.y);
      float b0 = q[0], pa = q[1];
      return f3(b0 * tanf(pa * p.y / r), -b0 * tanf(pa * p.x / r), b0);
    }
    case JSH_B_SPIRAL_CONICAL: {
      float bz = q[0] / (p.z * p.z);
      float tp = X.tan_pitch;
      return f3(bz * (p.x / p.z + p.y * tp), bz * (p.y / p.z - p.x * tp), bz);
    }
    case JSH_B_FORCE_FREE_CYLINDRICAL: {
      float s, c;
      sincos_atan(p.y / p.x, s, c);
      float b1 = X.b_bessel1;
      return f3(-b1 * s, b1 * s, X.b_bessel0);
    }
    case JSH_B_HELICAL_CONICAL: {
      float b = q[0] * fpow(sqrtf(fdot(p, p)), -q[1]);
      float rc2 = p.x * p.x + p.y * p.y;
      float px = 0.f, py = 0.f;
      if (rc2 > 0.f) {
        float irc = rsqrtf(rc2);
        px = -p.y * irc;
        py = p.x * irc;
        if (q[3] != 0.f && p.x < 0.f) {
          px = -px;
          py = -py;
        }
      }
      float bt = b * X.sin_pitch;
      return f3(bt * px, bt * py, b * X.cos_pitch);
    }
    case JSH_B_SIMULATION: {
      float s, c;
      sincos_atan(p.y / p.x, s, c);
      float bp = sim32(m.grids[0], m.fb_p, p, 0.f);
      float bphi = sim32(m.grids[0], m.fb_phi, p, 0.f);
      return f3(-s * bphi, c * bphi, bp);
    }
    default: return f3(0, 0, 0);
  }
}

// ------------------------------------------------------- random directions
// The cell nearest to p [pc] in FP32 (the lowest index among equal
// distances): the mixed path's own position is FP32, so a point within its
// rounding of a face between two cells may take either neighbour.
__device__ inline int cells_nearest32(const JshCells& C, F3 p) {
  const float fx = (p.x - C.x0f) * C.inv_hf, fy = (p.y - C.y0f) * C.inv_hf, fz = (p.z - C.z0f) * C.inv_hf;
  const bool inside = fx >= 0.f && fy >= 0.f && fz >= 0.f && fx < (float)C.nbx && fy < (float)C.nby &&
                      fz < (float)C.nbz;
  int q0 = 0, q1 = C.n;
  const int32_t* list = nullptr;
  if (inside) {
    const int b = (min((int)fz, C.nbz - 1) * C.nby + min((int)fy, C.nby - 1)) * C.nbx + min((int)fx, C.nbx - 1);
    q0 = C.bstart[b];
    q1 = C.bstart[b + 1];
    list = C.bitems;
  }
  float best = INFINITY;
  int bi = 0;
  for (int q = q0; q < q1; ++q) {
    const int c = list ? list[q] : q;
    const F3 d = p - f3(C.pf[3 * c], C.pf[3 * c + 1], C.pf[3 * c + 2]);
    const float d2 = fdot(d, d);
    if (d2 < best) {
      best = d2;
      bi = c;
    }
  }
  return bi;
}

// RandomVectorBField::bf (src/BField.cpp:154-161) in FP32: B + fraction |B| n
// with the nearest cell's direction or the per-evaluation draw of the key
// (pixel of hit h, frequency f, evaluation index e).
__device__ inline F3 brandom32(const JshRequest& R, F3 B, F3 p, uint32_t h, uint32_t f, uint32_t e) {
  const JshModel& m = R.model;
  F3 n;
  if (m.rnd_kind == JSH_RND_CELLS) {
    const int c = cells_nearest32(m.cells, p);
    n = f3(m.cells.dirf[3 * c], m.cells.dirf[3 * c + 1], m.cells.dirf[3 * c + 2]);
  } else {
    double nd[3];
    jsh_random_direction(m.rnd_seed, (uint32_t)R.hits[h].pix, f, e, nd);
    n = f3((float)nd[0], (float)nd[1], (float)nd[2]);
  }
  return B + n * ((float)m.rnd_frac * sqrtf(fdot(B, B)));
}

// ------------------------------------------------------- coefficients
struct Coef32 {
  float kI, kQ, kV, kF, kC, eI, eQ, eV;
};

// Kinematics of a (Gamma, v_hat) velocity for the LOS n (towards the
// observer): Doppler factor D and the aberrated LOS n' (src/utils.cpp:147-162).
__device__ __forceinline__ void kinematics32(float gamma, F3 vdir, F3 n, float& D, F3& nlp, float& beta) {
  float g2 = gamma * gamma;
  beta = sqrtf(fmaxf((gamma - 1.f) * (gamma + 1.f), 0.f)) / gamma;
  F3 dv = vdir - n;
  float one_m_bn = 1.f / (g2 * (1.f + beta)) + beta * 0.5f * fdot(dv, dv);
  D = 1.f / (gamma * one_m_bn);
  nlp = n * D - vdir * ((D + 1.f) * (gamma / (gamma + 1.f)) * beta);
}

// The coefficients from the plasma-frame density np_, field B, aberrated LOS
// nlp and Doppler factor D (the algebra of the file header).
__device__ __forceinline__ void coef32_tail(const JshFreqConst& F, const JshMixed& X, float np_, F3 B, F3 nlp,
                                            float D, bool full, Coef32& c) {
  F3 cr = fcross(nlp, B);
  float w = sqrtf(fdot(cr, cr)) * D;
  float P = 0.f, Rw = 0.f;
  // w = 0 (no field across the line of sight) gives zero coefficients; a
  // NaN field (a law undefined at the point) propagates as in the reference
  if (!(w <= 0.f)) {
    P = fpow(w, X.pk);
    Rw = P * rsqrtf(w);
  }
  c.kI = F.ak * np_ * P;
  c.eI = F.ae * np_ * Rw * D;
  if (!full) return;
  float bpar = fdot(B, nlp);
  c.kQ = X.kq * c.kI;
  c.eQ = X.eq * c.eI;
  c.kV = -F.av * np_ * bpar * Rw * D;
  c.eV = (w > 0.f) ? -F.aev * np_ * bpar * D * D * (P / w) : 0.f;
  c.kF = F.af * np_ * bpar * D;
  c.kC = -F.ac * np_ * (F.c1 * w * w - F.c2 * P);
}

// Which coefficients coef32_rt computes: k_I only (the tau pass), k_I and
// eta_I (I-only output), all of them.  k_I comes out bitwise the same in
// every mode, so an item's tau does not depend on the modes its warp-mates
// force on it.
enum CoefMode { COEF_KI = 0, COEF_I = 1, COEF_FULL = 2 };

// The benchmark family in the plasma frame (ConstFlat V, helical conical B,
// BK n) in the log domain: with l = log2|p|, u the helical unit direction
// and w = |n' x B| D = b |n' x u| D,
//   log2 n' = log2 n0' - m_n l,   log2 w = log2(b0 D) - m_b l + log2 |n' x u|,
//   k_I = a_k n' 2^(pk log2 w),  eta_I = a_e D n' 2^((pk - 1/2) log2 w)
// (pk = (s + 2) / 2): the tau pass's k_I costs two log2, one rsqrt and two
// exp2 instead of eight MUFU operations.  The other coefficients follow
// from k_I, eta_I, n', b and w: k_V = -(a_V / a_e) B_par eta_I, eta_V =
// -(a_eV / a_k) B_par D^2 k_I / w, k_F = a_F n' B_par D, k_C = -a_C c1 n' w^2
// + (a_C c2 / a_k) k_I, B_par = b (u . n').
__device__ __forceinline__ void coef32_helical_log(const JshMixed& X, const JshFreqConst& F, F3 p, int mode,
                                                   Coef32& c) {
  const float l = 0.5f * __log2f(fdot(p, p));
  const float rc2 = p.x * p.x + p.y * p.y;
  float px = 0.f, py = 0.f;
  if (rc2 > 0.f) {
    const float irc = rsqrtf(rc2);
    px = -p.y * irc;
    py = p.x * irc;
    if (X.bq[3] != 0.f && p.x < 0.f) {
      px = -px;
      py = -py;
    }
  }
  const float st = X.b_sign * X.sin_pitch;
  const F3 u = f3(st * px, st * py, X.b_sign * X.cos_pitch);
  const F3 nlp = f3(X.nlp[0], X.nlp[1], X.nlp[2]);
  const F3 cr = fcross(nlp, u);
  const float lw = fmaf(-X.bq[1], l, X.l2_b0D) + 0.5f * __log2f(fdot(cr, cr));
  // n' and w^pk as two exp2 of arguments of ~20 each rather than one of ~50:
  // exp2f's relative error is ~ulp(argument), so the split keeps k_I's
  // rounding at the level of the product form
  const float n_ = exp2f(fmaf(-X.nq[1], l, X.l2_n0));
  c.kI = (F.ak * n_) * exp2f(X.pk * lw);
  if (mode == COEF_KI) return;
  c.eI = (F.ae * X.D * n_) * exp2f(X.pk_h * lw);
  if (mode == COEF_I) return;
  const float bpar = exp2f(fmaf(-X.bq[1], l, X.l2_b0)) * fdot(u, nlp);
  const float w = exp2f(lw);
  const float D = X.D;
  c.kQ = X.kq * c.kI;
  c.eQ = X.eq * c.eI;
  c.kV = -F.r_kv * bpar * c.eI;
  c.eV = (w > 0.f) ? -F.r_ev * bpar * (D * D) * (c.kI / w) : 0.f;
  c.kF = F.af * n_ * bpar * D;
  c.kC = fmaf(F.r_kc, c.kI, -F.ac * F.c1 * n_ * (w * w));
}

// (rk_h, rk_f, rk_e): hit index, frequency and evaluation index of the
// per-evaluation random direction (JSH_RND_POINTS only); tri_hint: the
// lane's point-location hint for fields on one shared grid (may be null).
// GENERAL = false compiles the fused benchmark-family path alone, for
// kernels launched only on requests whose mix.helical_log is set (the same
// arithmetic as the general build takes for them).
template <bool GENERAL = true>
__device__ __forceinline__ void coef32_rt(const JshRequest& R, const JshFreqConst& F, F3 p, int mode, Coef32& c,
                                          uint32_t rk_h = 0, uint32_t rk_f = 0, uint32_t rk_e = 0,
                                          int* tri_hint = nullptr) {
  const JshModel& m = R.model;
  const JshMixed& X = R.mix;
  if (!GENERAL || X.helical_log) {
    coef32_helical_log(X, F, p, mode, c);
    return;
  }
  const bool full = mode == COEF_FULL;
  float D, gamma, beta, np_;
  F3 nlp, vdir, B;
  if (X.helical_bk) {
    // the benchmark family (ConstFlat V, helical conical B, BK n) fused: both
    // power laws of |p| from one log2, no kind dispatch
    D = X.D;
    gamma = X.gamma;
    beta = X.beta;
    nlp = f3(X.nlp[0], X.nlp[1], X.nlp[2]);
    vdir = f3(0, 0, 1);
    const float l2r = 0.5f * __log2f(fdot(p, p));
    const float n = X.nq[0] * exp2f(-X.nq[1] * l2r);
    np_ = m.n_plasma ? n : n / gamma;
    const float b = X.bq[0] * exp2f(-X.bq[1] * l2r);
    const float rc2 = p.x * p.x + p.y * p.y;
    float px = 0.f, py = 0.f;
    if (rc2 > 0.f) {
      const float irc = rsqrtf(rc2);
      px = -p.y * irc;
      py = p.x * irc;
      if (X.bq[3] != 0.f && p.x < 0.f) {
        px = -px;
        py = -py;
      }
    }
    const float bt = b * X.sin_pitch;
    B = f3(bt * px, bt * py, b * X.cos_pitch);
  } else if (X.sim_shared) {
    // every field from one grid (the simulation workload): one point location
    // for Gamma, n, B_p and B_phi
    const GridW g = grid_locate32(m.grids[0], p.z, sqrtf(p.x * p.x + p.y * p.y), tri_hint);
    gamma = grid_val32(m.grids[0], g, m.f_v, 1.0f);
    vdir = f3(0, 0, 1);
    kinematics32(gamma, vdir, f3(X.nl[0], X.nl[1], X.nl[2]), D, nlp, beta);
    const float n = grid_val32(m.grids[0], g, m.f_n, 0.f);
    np_ = m.n_plasma ? n : n / gamma;
    float s, cph;
    sincos_atan(p.y / p.x, s, cph);
    const float bp = grid_val32(m.grids[0], g, m.fb_p, 0.f);
    const float bphi = grid_val32(m.grids[0], g, m.fb_phi, 0.f);
    B = f3(-s * bphi, cph * bphi, bp);
  } else {
    if (X.v_const) {
      D = X.D;
      gamma = X.gamma;
      beta = X.beta;
      nlp = f3(X.nlp[0], X.nlp[1], X.nlp[2]);
      vdir = f3(0, 0, 1);
    } else {
      Vel v = vfield32(m, X, p);
      gamma = v.gamma;
      vdir = v.dir;
      kinematics32(gamma, vdir, f3(X.nl[0], X.nl[1], X.nl[2]), D, nlp, beta);
    }
    float n = nfield32(m, X, p);
    np_ = m.n_plasma ? n : n / gamma;
    if (m.b_scalar) {
      float w = bscalar32(m, X, p) * D;
      float P = fpow(w, X.pk);
      float Rw = P * rsqrtf(w);
      c.kI = F.ak * np_ * P;
      c.eI = F.ae * np_ * Rw * D;
      c.kQ = c.kV = c.kF = c.kC = c.eQ = c.eV = 0.f;
      return;
    }
    B = bvector32(m, X, p);
  }
  if (m.rnd_kind != JSH_RND_NONE) B = brandom32(R, B, p, rk_h, rk_f, rk_e);
  if (!m.b_plasma) {
    // B' = B / Gamma + Gamma beta^2 / (1 + Gamma) v_hat (v_hat . B)
    B = B * (1.f / gamma) + vdir * (gamma * beta * beta / (1.f + gamma) * fdot(vdir, B));
  }
  coef32_tail(F, X, np_, B, nlp, D, full, c);
}

}  // namespace jsh
