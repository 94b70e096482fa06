// jsh_transfer64.cuh -- the all-FP64 per-(ray, frequency) transfer on the
// device: tau pass front to back with the dense-output Dormand-Prince
// stepper stopping at tau_max (src/Observation.cpp:126-214), then the I or
// IQUV pass back to front with the controlled stepper of
// integrate_adaptive (src/Observation.cpp:242-308; the IQUV right-hand side
// of src/System.cpp:41-63).
//
// Dormand-Prince 5(4) tableau: Dormand & Prince (1980).  Dense output:
// Hairer, Norsett & Wanner, Solving ODEs I, II.6.  Step control as
// documented for Boost.Odeint's controlled_runge_kutta / default_error_checker
// (error = max_i |e_i| / (atol + rtol (|x_i| + |dt| |x'_i|)), decrease
// max(0.9 err^-1/3, 0.2), increase 0.9 max(err, 5^-5)^-1/5 when err < 0.5,
// 500 consecutive rejections abort) and integrate_adaptive's truncation of
// the last step to the interval end.
#pragma once

#include <float.h>

#include "jsh_fields.cuh"
#include "jsh_request.h"

namespace jsh {

namespace dp {
constexpr double C2 = 1.0 / 5, C3 = 3.0 / 10, C4 = 4.0 / 5, C5 = 8.0 / 9;
constexpr double A21 = 1.0 / 5;
constexpr double A31 = 3.0 / 40, A32 = 9.0 / 40;
constexpr double A41 = 44.0 / 45, A42 = -56.0 / 15, A43 = 32.0 / 9;
constexpr double A51 = 19372.0 / 6561, A52 = -25360.0 / 2187, A53 = 64448.0 / 6561, A54 = -212.0 / 729;
constexpr double A61 = 9017.0 / 3168, A62 = -355.0 / 33, A63 = 46732.0 / 5247, A64 = 49.0 / 176,
                 A65 = -5103.0 / 18656;
constexpr double B1 = 35.0 / 384, B3 = 500.0 / 1113, B4 = 125.0 / 192, B5 = -2187.0 / 6784, B6 = 11.0 / 84;
constexpr double E1 = 71.0 / 57600, E3 = -71.0 / 16695, E4 = 71.0 / 1920, E5 = -17253.0 / 339200,
                 E6 = 22.0 / 525, E7 = -1.0 / 40;
constexpr double D1 = -12715105075.0 / 11282082432.0, D3 = 87487479700.0 / 32700410799.0,
                 D4 = -10690763975.0 / 1880347072.0, D5 = 701980252875.0 / 199316789632.0,
                 D6 = -1453857185.0 / 822651844.0, D7 = 69997945.0 / 29380423.0;
constexpr int FAIL_LIMIT = 500;
}  // namespace dp

// Tableau rows of stages 2..7 (row 7 = the 5th-order weights b) and nodes.
__device__ __forceinline__ double dp_a(int s, int j) {
  switch (s * 8 + j) {
    case 8: return dp::A21;
    case 16: return dp::A31;
    case 17: return dp::A32;
    case 24: return dp::A41;
    case 25: return dp::A42;
    case 26: return dp::A43;
    case 32: return dp::A51;
    case 33: return dp::A52;
    case 34: return dp::A53;
    case 35: return dp::A54;
    case 40: return dp::A61;
    case 41: return dp::A62;
    case 42: return dp::A63;
    case 43: return dp::A64;
    case 44: return dp::A65;
    case 48: return dp::B1;
    case 50: return dp::B3;
    case 51: return dp::B4;
    case 52: return dp::B5;
    case 53: return dp::B6;
    default: return 0.0;
  }
}
__device__ __forceinline__ double dp_c(int s) {
  switch (s) {
    case 1: return dp::C2;
    case 2: return dp::C3;
    case 3: return dp::C4;
    case 4: return dp::C5;
    default: return 1.0;
  }
}

__device__ __forceinline__ double dt_decrease(double dt, double err, double max_dt) {
  double f = 0.9 * pow(err, -1.0 / 3.0);
  dt *= (f > 0.2 ? f : 0.2);
  if (max_dt != 0.0 && fabs(dt) > max_dt) dt = max_dt;
  return dt;
}

__device__ __forceinline__ double dt_increase(double dt, double err, double max_dt) {
  if (err < 0.5) {
    const double lo = 0.00032;  // 5^-5
    double e = err > lo ? err : lo;
    dt *= 9.0 / 10.0 * pow(e, -1.0 / 5.0);
    if (max_dt != 0.0 && fabs(dt) > max_dt) dt = max_dt;
  }
  return dt;
}

// Right-hand sides.  Path point(t) = p0 + t * dir; nl = LOS towards the observer.
struct Path64 {
  D3 p0, dir, nl;
  double nu;
  uint32_t rk0, rk1;  // random-direction key of the item: pixel, frequency
  uint32_t* ev;       // the item's evaluation counter (NULL: key index 0)
};

template <int DIM, bool FULL>
struct Rhs64 {
  // TAU (DIM == 1, !FULL used as tau):  dtau/dt = kI
  __device__ __forceinline__ static void eval(const JshModel& m, const Path64& P, bool tau, double t,
                                              const double* x, double* dx) {
    D3 p = P.p0 + P.dir * t;
    double k[NCOEF];
    const uint32_t ev = P.ev ? (*P.ev)++ : 0u;
    if (tau) {
      coefficients64<false>(m, p, P.nl, P.nu, k, P.rk0, P.rk1, ev);
      dx[0] = k[CK_I];
      return;
    }
    coefficients64<FULL>(m, p, P.nl, P.nu, k, P.rk0, P.rk1, ev);
    if (!FULL) {
      dx[0] = k[CE_I] - k[CK_I] * x[0];
      return;
    }
    dx[0] = k[CE_I] - k[CK_I] * x[0] - k[CK_Q] * x[1] - k[CK_V] * x[3];
    dx[1] = k[CE_Q] - k[CK_I] * x[1] - k[CK_Q] * x[0] - k[CK_F] * x[2];
    dx[2] = -k[CK_I] * x[2] + k[CK_F] * x[1] - k[CK_C] * x[3];
    dx[3] = k[CE_V] - k[CK_I] * x[3] - k[CK_V] * x[0] + k[CK_C] * x[2];
  }
};

struct Ctl64 {
  double atol, rtol, max_dt;
  int64_t max_steps;
  uint64_t acc, rej, evals;
};

// One successful controlled step from (t, x) with FSAL derivative k[0];
// retries rejected attempts.  On success x, t advance, dt is the proposal for
// the next step, k1_old/x_old/dt_used describe the accepted step for dense
// output and k[0] holds the new FSAL derivative.  Returns 0 or a status bit.
template <int DIM, bool FULL>
__device__ uint32_t controlled_step64(const JshModel& m, const Path64& P, bool tau, Ctl64& C, double& t, double* x,
                                      double& dt, double (&k)[7][DIM], double* x_old, double* k1_old,
                                      double& dt_used, int64_t& nsteps) {
  using R = Rhs64<DIM, FULL>;
  int fails = 0;
  for (;;) {
    if (nsteps++ >= C.max_steps) return JSH_ST_STEP_LIMIT;
    if (C.max_dt != 0.0 && fabs(dt) > C.max_dt) {
      dt = C.max_dt;
      C.rej++;
      if (++fails >= dp::FAIL_LIMIT) return JSH_ST_FAIL_LIMIT;
      continue;
    }
    // stages 2..7 as a loop over the tableau (one right-hand-side call site);
    // row 7 is the 5th-order solution, whose derivative is the FSAL stage
    double y[DIM], xn[DIM];
#pragma unroll 1
    for (int s = 1; s < 7; ++s) {
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
        double acc = dp_a(s, 0) * k[0][i];
        for (int j = 1; j < s; ++j) acc += dp_a(s, j) * k[j][i];
        y[i] = x[i] + dt * acc;
      }
      R::eval(m, P, tau, t + dp_c(s) * dt, y, k[s]);
    }
#pragma unroll
    for (int i = 0; i < DIM; ++i) xn[i] = y[i];
    C.evals += 6;
    double e = 0.0;
    bool bad = false;
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      double err = dt * (dp::E1 * k[0][i] + dp::E3 * k[2][i] + dp::E4 * k[3][i] + dp::E5 * k[4][i] +
                         dp::E6 * k[5][i] + dp::E7 * k[6][i]);
      double r = fabs(err) / (C.atol + C.rtol * (fabs(x[i]) + fabs(dt) * fabs(k[0][i])));
      bad |= isnan(r);
      e = r > e ? r : e;
    }
    if (bad) return JSH_ST_NAN;
    if (e > 1.0) {
      dt = dt_decrease(dt, e, C.max_dt);
      C.rej++;
      if (++fails >= dp::FAIL_LIMIT) return JSH_ST_FAIL_LIMIT;
      continue;
    }
    double t_new = t + dt;
    if (t_new == t) return JSH_ST_DT_UNDERFLOW;
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      x_old[i] = x[i];
      x[i] = xn[i];
      k1_old[i] = k[0][i];
      k[0][i] = k[6][i];
    }
    dt_used = dt;
    t = t_new;
    dt = dt_increase(dt, e, C.max_dt);
    C.acc++;
    return 0;
  }
}

// steps_schedule (src/utils.cpp:354-366) with its default tau limits.
__device__ __forceinline__ int steps_schedule(double tau, int n_min, int n_max) {
  const double tau_min = 0.1, tau_max = 100.0;
  if (tau <= tau_min) return n_min;
  if (tau >= tau_max) return n_max;
  double b = -log(tau_min);
  double k = n_max / pow((log(tau_max) + b), 2.0);
  double n = k * pow((log(tau) + b), 2.0) + n_min;
  return (int)ceil(n);
}

struct ItemOut {
  double tau, l, iquv[4];
  uint32_t status;
};

// The transfer of one hit ray at one frequency.
template <bool FULL>
__device__ void transfer_item64(const JshModel& m, const JshPlane& pl, const JshParamsDev& Pp, const JshHit& hit,
                                double nu, int f, ItemOut& o, Ctl64& tot) {
  uint32_t ev = 0;  // evaluation index of the item (random-direction key)
  o.tau = o.l = 0.0;
  o.iquv[0] = o.iquv[1] = o.iquv[2] = o.iquv[3] = 0.0;
  o.status = (uint32_t)hit.status | JSH_ST_HIT;
  const int64_t max_steps = Pp.max_steps > 0 ? Pp.max_steps : ((int64_t)1 << 22);
  D3 rd = d3(pl.dx, pl.dy, pl.dz);
  D3 rd2 = d3(pl.rx, pl.ry, pl.rz);
  D3 nl = rd * -1.;
  double seg[JSH_MAX_SEG][6];
  int nseg = hit.nseg;
#pragma unroll
  for (int s = 0; s < JSH_MAX_SEG; ++s)
#pragma unroll
    for (int q = 0; q < 6; ++q) seg[s][q] = hit.seg[s][q];

  // ---- tau pass ----
  double background_tau = 0.0, thickness = 0.0;
  for (int sidx = 0; sidx < nseg; ++sidx) {
    D3 pin = d3(seg[sidx][0], seg[sidx][1], seg[sidx][2]);
    D3 pout = d3(seg[sidx][3], seg[sidx][4], seg[sidx][5]);
    D3 dd = pout - pin;
    double length = sqrt((dd.x * dd.x + dd.y * dd.y) + dd.z * dd.z);
    double dt = length / Pp.n;
    Path64 P{pin, rd, nl, nu, (uint32_t)hit.pix, (uint32_t)f, &ev};
    Ctl64 C{Pp.tau_atol, Pp.tau_rtol, Pp.dt_max, max_steps, 0, 0, 0};
    double t = 0.0, x[1] = {0.0}, k[7][1], x_old[1] = {0.0}, k1_old[1] = {0.0}, dt_used = 0.0, t_old = 0.0;
    bool init = false, crossed = false;
    int64_t nsteps = 0;
    uint32_t fail = 0;
    while (length - t > DBL_EPSILON) {
      if ((t + dt) - length > DBL_EPSILON) dt = length - t;
      if (!init) {
        Rhs64<1, false>::eval(m, P, true, t, x, k[0]);
        C.evals++;
        init = true;
      }
      t_old = t;
      fail = controlled_step64<1, false>(m, P, true, C, t, x, dt, k, x_old, k1_old, dt_used, nsteps);
      if (fail) break;
      if (x[0] >= Pp.tau_max) {
        crossed = true;
        break;
      }
    }
    tot.evals += C.evals;
    tot.acc += C.acc;
    tot.rej += C.rej;
    if (fail) {
      o.status |= fail;
      o.tau = background_tau + x[0];
      o.l = thickness + length;
      return;
    }
    if (crossed) {
      o.status |= JSH_ST_TAU_CROSSED;
      double t0 = t_old, t1 = t, xm = x[0], t_m;
      int it = 0;
      while (fabs(xm - Pp.tau_max) > Pp.tau_precision) {
        if (++it > 200) {
          o.status |= JSH_ST_BISECT_LIMIT;
          break;
        }
        t_m = 0.5 * (t0 + t1);
        double theta = (t_m - t_old) / dt_used, th1 = 1.0 - theta;
        double ydiff = x[0] - x_old[0];
        double bspl = dt_used * k1_old[0] - ydiff;
        double r4 = ydiff - dt_used * k[6][0] - bspl;
        double r5 = dt_used * (dp::D1 * k1_old[0] + dp::D3 * k[2][0] + dp::D4 * k[3][0] + dp::D5 * k[4][0] +
                               dp::D6 * k[5][0] + dp::D7 * k[6][0]);
        xm = x_old[0] + theta * (ydiff + th1 * (bspl + theta * (r4 + th1 * r5)));
        if (xm > Pp.tau_max) t1 = t_m;
        else t0 = t_m;
      }
      t_m = 0.5 * (t0 + t1);
      D3 po = pin + rd2 * t_m;
      seg[sidx][3] = po.x;
      seg[sidx][4] = po.y;
      seg[sidx][5] = po.z;
      nseg = sidx + 1;
    }
    background_tau += x[0];
    thickness += length;
    if (crossed) break;
  }
  o.tau = background_tau;
  o.l = thickness;
  if (!(background_tau > Pp.tau_min)) return;
  o.status |= JSH_ST_IQUV;

  // ---- I / IQUV pass ----
  constexpr int DIM = FULL ? 4 : 1;
  double st[DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i) st[i] = 0.0;
  for (int sidx = nseg - 1; sidx >= 0; --sidx) {
    D3 pin = d3(seg[sidx][0], seg[sidx][1], seg[sidx][2]);
    D3 pout = d3(seg[sidx][3], seg[sidx][4], seg[sidx][5]);
    D3 dd = pout - pin;
    double length = sqrt((dd.x * dd.x + dd.y * dd.y) + dd.z * dd.z);
    double auto_n = Pp.n;
    if (background_tau > 0.1) auto_n = steps_schedule(background_tau, Pp.n, 10 * Pp.n);
    double dt = length / auto_n;
    Path64 P{pout, nl, nl, nu, (uint32_t)hit.pix, (uint32_t)f, &ev};
    Ctl64 C{Pp.atol, Pp.rtol, 0.0, max_steps, 0, 0, 0};
    double t = 0.0, k[7][DIM], x_old[DIM], k1_old[DIM], dt_used;
    int64_t nsteps = 0;
    uint32_t fail = 0;
    bool first = true;
    while (length - t > DBL_EPSILON) {
      if ((t + dt) - length > DBL_EPSILON) dt = length - t;
      if (first) {
        Rhs64<DIM, FULL>::eval(m, P, false, t, st, k[0]);
        C.evals++;
        first = false;
      }
      fail = controlled_step64<DIM, FULL>(m, P, false, C, t, st, dt, k, x_old, k1_old, dt_used, nsteps);
      if (fail) break;
    }
    tot.evals += C.evals;
    tot.acc += C.acc;
    tot.rej += C.rej;
    if (fail) {
      o.status |= fail;
      break;
    }
  }
#pragma unroll
  for (int i = 0; i < DIM; ++i) o.iquv[i] = st[i];
}

}  // namespace jsh
