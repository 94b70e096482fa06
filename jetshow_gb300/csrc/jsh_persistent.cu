// jsh_persistent.cu -- the mixed-precision transfer: FP32 right-hand sides
// and Runge-Kutta stages; FP64 time, step size, error-control arithmetic,
// accumulated optical depth and Faraday rotation angle.  One work item is a
// (request, hit ray, frequency); its tau pass (src/Observation.cpp:126-214)
// and I/IQUV pass (src/Observation.cpp:242-308, src/System.cpp:41-63) run
// as a per-lane state machine that advances by one Dormand-Prince attempt
// per call, so that
//  * the static schedule runs one item per thread to completion, and
//  * the persistent schedule keeps every warp busy: lanes whose ray has
//    finished are refilled from a global work queue (warp ballot + popc
//    rank, one atomic per warp) while the other lanes keep stepping.
//
// The IQUV state is integrated in a frame rotating with the Faraday angle
// chi (dchi/dt = k_F): with (Q, U) = R(chi) (q, u) the k_F terms of the
// reference right-hand side cancel and
//   dI/dt = eta_I - k_I I - k_Q (c q - s u) - k_V V
//   dq/dt = -k_I q + c (eta_Q - k_Q I) - s k_C V
//   du/dt = -k_I u - s (eta_Q - k_Q I) - c k_C V
//   dV/dt = eta_V - k_I V - k_V I + k_C (s q + c u),   c, s = cos, sin chi.
// chi accumulates in FP64; each stage rotates by the FP32 increment.  The
// error norm adds |err_chi| * |P| as the polarised-intensity error of the
// rotation.  Intensities are scaled by a per-frequency power of two and
// lengths are in pc so the FP32 state stays well inside its range.
#include <float.h>
#include <math.h>

#include "jsh_batch.cuh"
#include "jsh_context.h"
#include "jsh_fields.cuh"
#include "jsh_fields32.cuh"
#include "jsh_launch.h"
#include "jsh_transfer64.cuh"

namespace jsh {

namespace {

constexpr uint8_t PH_IDLE = 0, PH_TAU = 1, PH_IQUV = 2;
constexpr double INV_PC = 1.0 / JSH_PC;

struct Lane {
  int r, f;
  uint32_t h;
  uint8_t phase;
  int8_t seg, nseg;
  bool init, trunc;
  double p0x, p0y, p0z;  // segment start [pc]
  double length;         // [pc]
  double length_cm;
  double t, dt;          // [pc]
  double tau_seg, tau_bg, thick;
  double t_cross;        // [pc] tau_max point on the last tau segment
  double chi;
  float x[4];
  float k1[5];
  int32_t nsteps, fails;
  uint32_t status;
  uint32_t evals, acc, rej;
};

__device__ __forceinline__ double seg_len_cm(const JshHit& H, int s, double ox, double oy, double oz) {
  double dx = ox - H.seg[s][0], dy = oy - H.seg[s][1], dz = oz - H.seg[s][2];
  return sqrt((dx * dx + dy * dy) + dz * dz);
}

__device__ __forceinline__ void begin_tau_segment(Lane& L, const JshRequest& R, const JshHit& H) {
  int s = L.seg;
  L.length_cm = seg_len_cm(H, s, H.seg[s][3], H.seg[s][4], H.seg[s][5]);
  L.length = L.length_cm * INV_PC;
  L.p0x = H.seg[s][0] * INV_PC;
  L.p0y = H.seg[s][1] * INV_PC;
  L.p0z = H.seg[s][2] * INV_PC;
  L.t = 0.0;
  L.dt = L.length / R.P.n;
  L.tau_seg = 0.0;
  L.init = false;
  L.nsteps = 0;
  L.fails = 0;
}

__device__ __forceinline__ void begin_iquv_segment(Lane& L, const JshRequest& R, const JshHit& H) {
  int s = L.seg;
  double ox = H.seg[s][3], oy = H.seg[s][4], oz = H.seg[s][5];
  if (L.trunc && s == L.nseg - 1) {
    double tc = L.t_cross * JSH_PC;
    ox = H.seg[s][0] + R.plane.rx * tc;
    oy = H.seg[s][1] + R.plane.ry * tc;
    oz = H.seg[s][2] + R.plane.rz * tc;
  }
  L.length_cm = seg_len_cm(H, s, ox, oy, oz);
  L.length = L.length_cm * INV_PC;
  L.p0x = ox * INV_PC;
  L.p0y = oy * INV_PC;
  L.p0z = oz * INV_PC;
  double auto_n = R.P.n;
  if (L.tau_bg > 0.1) auto_n = steps_schedule(L.tau_bg, R.P.n, 10 * R.P.n);
  L.t = 0.0;
  L.dt = L.length / auto_n;
  L.init = false;
  L.nsteps = 0;
  L.fails = 0;
}

__device__ __forceinline__ void lane_start(Lane& L, const JshRequest* __restrict__ reqs,
                                           const unsigned long long* base, int n_req, unsigned long long w) {
  int r = find_request(base, n_req, w);
  const JshRequest& R = reqs[r];
  unsigned long long local = w - base[r];
  unsigned nhit = *R.n_hit;
  L.r = r;
  L.f = (int)(local / nhit);
  L.h = (uint32_t)(local % nhit);
  const JshHit& H = R.hits[L.h];
  L.phase = PH_TAU;
  L.seg = 0;
  L.nseg = (int8_t)H.nseg;
  L.trunc = false;
  L.tau_bg = 0.0;
  L.thick = 0.0;
  L.t_cross = -1.0;
  L.chi = 0.0;
  L.x[0] = L.x[1] = L.x[2] = L.x[3] = 0.f;
  L.status = (uint32_t)H.status | JSH_ST_HIT;
  L.evals = L.acc = L.rej = 0;
  begin_tau_segment(L, R, H);
}

__device__ __forceinline__ void lane_finish(Lane& L, const JshRequest* __restrict__ reqs) {
  const JshRequest& R = reqs[L.r];
  const JshHit& H = R.hits[L.h];
  const JshFreqConst& F = R.mix.fc[L.f];
  uint64_t q = (uint64_t)L.f * R.npix + (uint64_t)H.pix;
  double S = F.scale;
  double sc, ss;
  sincos(L.chi, &ss, &sc);
  double qq = L.x[1], uu = L.x[2];
  if (R.tau) R.tau[q] = L.tau_bg;
  if (R.l) R.l[q] = L.thick;
  if (R.I) R.I[q] = S * (double)L.x[0];
  if (R.Q) R.Q[q] = S * (sc * qq - ss * uu);
  if (R.U) R.U[q] = S * (ss * qq + sc * uu);
  if (R.V) R.V[q] = S * (double)L.x[3];
  if (R.status) R.status[q] = L.status;
  unsigned long long* c = R.counters;
  atomicAdd(&c[0], (unsigned long long)L.evals);
  atomicAdd(&c[1], (unsigned long long)L.acc);
  atomicAdd(&c[2], (unsigned long long)L.rej);
  atomicOr(&c[3], (unsigned long long)L.status);
  L.phase = PH_IDLE;
}

// Right-hand side at a stage.  tau: dk[0] = k_I.  IQUV: the rotating-frame
// system above; dk[4] = k_F = dchi/dt.
template <bool FULL>
__device__ __forceinline__ void rhs32(const JshRequest& R, const JshFreqConst& F, bool tau, bool tau_coef_only,
                                      F3 p, const float* y, float cs, float sn, float* dk) {
  Coef32 c;
  if (tau_coef_only || !FULL) coef32<false>(R, F, p, c);
  else coef32<true>(R, F, p, c);
  if (tau) {
    dk[0] = c.kI;
    if (FULL) dk[1] = dk[2] = dk[3] = dk[4] = 0.f;
    return;
  }
  if (!FULL) {
    dk[0] = c.eI - c.kI * y[0];
    return;
  }
  float Qlab = cs * y[1] - sn * y[2];
  float Ulab = sn * y[1] + cs * y[2];
  float sQ = c.eQ - c.kQ * y[0];
  float sU = -c.kC * y[3];
  dk[0] = c.eI - c.kI * y[0] - c.kQ * Qlab - c.kV * y[3];
  dk[1] = -c.kI * y[1] + cs * sQ + sn * sU;
  dk[2] = -c.kI * y[2] - sn * sQ + cs * sU;
  dk[3] = c.eV - c.kI * y[3] - c.kV * y[0] + c.kC * Ulab;
  dk[4] = c.kF;
}

// One Dormand-Prince attempt (or a phase transition) of an active lane.
// warp_tau: every active lane of the warp is in its tau pass, so only k_I
// is evaluated.
template <bool FULL>
__device__ __forceinline__ void lane_step(Lane& L, const JshRequest* __restrict__ reqs, bool warp_tau) {
  constexpr int NK = FULL ? 5 : 1;
  const JshRequest& R = reqs[L.r];
  const JshFreqConst F = R.mix.fc[L.f];
  const bool tau = (L.phase == PH_TAU);
  const bool coef_tau_only = tau && warp_tau;
  const double sgn = tau ? 1.0 : -1.0;
  const double ddx = sgn * R.plane.dx, ddy = sgn * R.plane.dy, ddz = sgn * R.plane.dz;
  const F3 dirf = f3((float)ddx, (float)ddy, (float)ddz);
  const double max_dt = tau ? R.mix.dt_max_pc : 0.0;
  // error-norm tolerances in FP32 (the norm needs a few digits; t and dt stay FP64)
  const float atol = tau ? (float)R.P.tau_atol : (float)F.atol;
  const float rtol = tau ? (float)R.P.tau_rtol : (float)R.P.rtol;

  // integrate_adaptive / adaptive range: finish at exactly t = length
  if (!(L.length - L.t > DBL_EPSILON)) goto segment_done;
  if ((L.t + L.dt) - L.length > DBL_EPSILON) L.dt = L.length - L.t;
  if (L.nsteps++ >= R.P.max_steps) {
    L.status |= JSH_ST_STEP_LIMIT;
    goto abort;
  }
  if (max_dt != 0.0 && fabs(L.dt) > max_dt) {
    L.dt = max_dt;
    L.rej++;
    if (++L.fails >= dp::FAIL_LIMIT) {
      L.status |= JSH_ST_FAIL_LIMIT;
      goto abort;
    }
    return;
  }
  {
    const F3 pn = f3((float)(L.p0x + L.t * ddx), (float)(L.p0y + L.t * ddy), (float)(L.p0z + L.t * ddz));
    // rotation of the frame at the step start: chi reduced modulo 2 pi in FP64
    // (3 FP64 operations), then an FP32 sincos of the reduced angle
    float c0 = 1.f, s0 = 0.f;
    if (FULL && !tau) {
      const double two_pi = 6.283185307179586;
      const float chr = (float)fma(-two_pi, rint(L.chi * (1.0 / two_pi)), L.chi);
      sincosf(chr, &s0, &c0);
    }
    if (!L.init) {
      rhs32<FULL>(R, F, tau, coef_tau_only, pn, L.x, c0, s0, L.k1);
      L.evals++;
      L.init = true;
    }
    const float h = (float)L.dt;
    float k[7][NK];
#pragma unroll
    for (int c = 0; c < NK; ++c) k[0][c] = L.k1[c];
    float y[4];
    auto stage = [&](int i, float cfrac, const float* a) {
      // y = x + h * sum_j a_j k_j ; rotation increment from the k_F column
#pragma unroll
      for (int c = 0; c < (FULL ? 4 : 1); ++c) {
        float acc = 0.f;
#pragma unroll
        for (int j = 0; j < 6; ++j)
          if (j < i) acc = fmaf(a[j], k[j][c], acc);
        y[c] = fmaf(h, acc, L.x[c]);
      }
      float cs = c0, sn2 = s0;
      if (FULL && !tau) {
        float d = 0.f;
#pragma unroll
        for (int j = 0; j < 6; ++j)
          if (j < i) d = fmaf(a[j], k[j][NK - 1], d);
        float sd, cd;
        __sincosf(h * d, &sd, &cd);
        cs = c0 * cd - s0 * sd;
        sn2 = s0 * cd + c0 * sd;
      }
      rhs32<FULL>(R, F, tau, coef_tau_only, pn + dirf * (cfrac * h), y, cs, sn2, k[i]);
    };
    const float a2[6] = {(float)dp::A21, 0, 0, 0, 0, 0};
    const float a3[6] = {(float)dp::A31, (float)dp::A32, 0, 0, 0, 0};
    const float a4[6] = {(float)dp::A41, (float)dp::A42, (float)dp::A43, 0, 0, 0};
    const float a5[6] = {(float)dp::A51, (float)dp::A52, (float)dp::A53, (float)dp::A54, 0, 0};
    const float a6[6] = {(float)dp::A61, (float)dp::A62, (float)dp::A63, (float)dp::A64, (float)dp::A65, 0};
    const float a7[6] = {(float)dp::B1, 0, (float)dp::B3, (float)dp::B4, (float)dp::B5, (float)dp::B6};
    stage(1, (float)dp::C2, a2);
    stage(2, (float)dp::C3, a3);
    stage(3, (float)dp::C4, a4);
    stage(4, (float)dp::C5, a5);
    stage(5, 1.0f, a6);
    stage(6, 1.0f, a7);
    L.evals += 6;
    // 5th-order increments and the embedded error estimate
    float inc[NK], err[NK];
#pragma unroll
    for (int c = 0; c < NK; ++c) {
      inc[c] = h * ((float)dp::B1 * k[0][c] + (float)dp::B3 * k[2][c] + (float)dp::B4 * k[3][c] +
                    (float)dp::B5 * k[4][c] + (float)dp::B6 * k[5][c]);
      err[c] = h * ((float)dp::E1 * k[0][c] + (float)dp::E3 * k[2][c] + (float)dp::E4 * k[3][c] +
                    (float)dp::E5 * k[4][c] + (float)dp::E6 * k[5][c] + (float)dp::E7 * k[6][c]);
    }
    // odeint default error checker: max_i |err_i| / (atol + rtol (|x_i| + |dt| |x'_i|))
    const float adt = fabsf(h);
    float e;
    if (tau) {
      e = fabsf(err[0]) / fmaf(rtol, fmaf(adt, fabsf(k[0][0]), fabsf((float)L.tau_seg)), atol);
    } else {
      e = 0.f;
#pragma unroll
      for (int c = 0; c < (FULL ? 4 : 1); ++c) {
        float r = fabsf(err[c]) / fmaf(rtol, fmaf(adt, fabsf(k[0][c]), fabsf(L.x[c])), atol);
        e = fmaxf(e, r);
      }
      if (FULL) {
        float P = sqrtf(fmaf(L.x[1], L.x[1], L.x[2] * L.x[2]));
        e = fmaxf(e, fabsf(err[NK - 1]) * P / fmaf(rtol, P, atol));
      }
    }
    if (!(e == e) || isinf(e)) {
      L.status |= JSH_ST_NAN;
      goto abort;
    }
    if (e > 1.0f) {
      float f = 0.9f * __powf(e, -1.0f / 3.0f);
      L.dt *= (double)(f > 0.2f ? f : 0.2f);
      if (max_dt != 0.0 && fabs(L.dt) > max_dt) L.dt = max_dt;
      L.rej++;
      if (++L.fails >= dp::FAIL_LIMIT) {
        L.status |= JSH_ST_FAIL_LIMIT;
        goto abort;
      }
      return;
    }
    // accept
    const double t_old = L.t, dt_used = L.dt;
    const double t_new = L.t + L.dt;
    if (t_new == L.t) {
      L.status |= JSH_ST_DT_UNDERFLOW;
      goto abort;
    }
    L.t = t_new;
    L.fails = 0;
    L.acc++;
    if (e < 0.5f) {
      float ee = e > 0.00032f ? e : 0.00032f;
      L.dt *= (double)(0.9f * __powf(ee, -0.2f));
      if (max_dt != 0.0 && fabs(L.dt) > max_dt) L.dt = max_dt;
    }
#pragma unroll
    for (int c = 0; c < NK; ++c) L.k1[c] = k[6][c];
    if (tau) {
      const double tau_old = L.tau_seg;
      L.tau_seg = tau_old + (double)inc[0];
      if (L.tau_seg >= R.P.tau_max) {
        // bisection on the dense output of this step (src/Observation.cpp:166-190)
        L.status |= JSH_ST_TAU_CROSSED;
        const float ydiff = inc[0];
        const float bspl = h * k[0][0] - ydiff;
        const float r4 = ydiff - h * k[6][0] - bspl;
        const float r5 = h * ((float)dp::D1 * k[0][0] + (float)dp::D3 * k[2][0] + (float)dp::D4 * k[3][0] +
                              (float)dp::D5 * k[4][0] + (float)dp::D6 * k[5][0] + (float)dp::D7 * k[6][0]);
        double t0 = t_old, t1 = t_new, xm = L.tau_seg, tm;
        int it = 0;
        while (fabs(xm - R.P.tau_max) > R.P.tau_precision) {
          if (++it > 200) {
            L.status |= JSH_ST_BISECT_LIMIT;
            break;
          }
          tm = 0.5 * (t0 + t1);
          float th = (float)((tm - t_old) / dt_used), th1 = 1.f - th;
          xm = tau_old + (double)(th * (ydiff + th1 * (bspl + th * (r4 + th1 * r5))));
          if (xm > R.P.tau_max) t1 = tm;
          else t0 = tm;
        }
        L.t_cross = 0.5 * (t0 + t1);
        L.trunc = true;
        L.nseg = L.seg + 1;
        L.tau_bg += L.tau_seg;
        L.thick += L.length_cm;
        goto start_iquv;
      }
    } else {
#pragma unroll
      for (int c = 0; c < (FULL ? 4 : 1); ++c) L.x[c] += inc[c];
      if (FULL) L.chi += (double)inc[NK - 1];
    }
    return;
  }

segment_done : {
  const JshHit& H = R.hits[L.h];
  if (tau) {
    L.tau_bg += L.tau_seg;
    L.thick += L.length_cm;
    if (L.seg + 1 < L.nseg) {
      L.seg++;
      begin_tau_segment(L, R, H);
      return;
    }
    goto start_iquv;
  }
  if (L.seg > 0) {
    L.seg--;
    begin_iquv_segment(L, R, H);
    return;
  }
  lane_finish(L, reqs);
  return;
}

start_iquv : {
  if (!(L.tau_bg > R.P.tau_min)) {
    lane_finish(L, reqs);
    return;
  }
  L.status |= JSH_ST_IQUV;
  L.phase = PH_IQUV;
  L.seg = L.nseg - 1;
  begin_iquv_segment(L, R, R.hits[L.h]);
  return;
}

abort:
  if (tau) {
    L.tau_bg += L.tau_seg;
    L.thick += L.length_cm;
  }
  lane_finish(L, reqs);
}

// One thread per work item, stepped to completion.
template <bool FULL>
__global__ void __launch_bounds__(128) transfer_static_mixed_kernel(const JshRequest* __restrict__ reqs,
                                                                     int n_req) {
  __shared__ unsigned long long base[JSH_MAX_BATCH + 1];
  batch_prefix(reqs, n_req, base);
  unsigned long long w = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= base[n_req]) return;
  Lane L;
  lane_start(L, reqs, base, n_req, w);
  while (L.phase != PH_IDLE) lane_step<FULL>(L, reqs, L.phase == PH_TAU);
}

// Persistent CTAs: each warp keeps 32 lanes busy, refilling idle lanes from
// the global queue when at least `refill` of them are idle.
template <bool FULL>
__global__ void __launch_bounds__(256) transfer_persistent_mixed_kernel(const JshRequest* __restrict__ reqs,
                                                                         int n_req, unsigned long long* queue,
                                                                         int refill) {
  __shared__ unsigned long long base[JSH_MAX_BATCH + 1];
  batch_prefix(reqs, n_req, base);
  const unsigned long long total = base[n_req];
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  Lane L;
  L.phase = PH_IDLE;
  bool exhausted = false;
  for (;;) {
    unsigned idle = __ballot_sync(0xffffffffu, L.phase == PH_IDLE);
    int nidle = __popc(idle);
    if (!exhausted && (nidle >= refill || nidle == 32) && nidle > 0) {
      unsigned long long b = 0;
      if (lane == 0) b = atomicAdd(queue, (unsigned long long)nidle);
      b = __shfl_sync(0xffffffffu, b, 0);
      if (b + (unsigned long long)nidle >= total) exhausted = true;
      if (L.phase == PH_IDLE) {
        unsigned long long w = b + (unsigned long long)__popc(idle & lt_mask);
        if (w < total) lane_start(L, reqs, base, n_req, w);
      }
    }
    unsigned active = __ballot_sync(0xffffffffu, L.phase != PH_IDLE);
    if (active == 0) {
      if (exhausted) break;
      continue;
    }
    bool warp_tau = __all_sync(0xffffffffu, L.phase != PH_IQUV);
    if (L.phase != PH_IDLE) lane_step<FULL>(L, reqs, warp_tau);
  }
}

}  // namespace


}  // namespace jsh

using namespace jsh;

cudaError_t jsh_launch_transfer_mixed(const JshRequest* d_reqs, int n_req, int schedule, bool full,
                                      uint64_t max_items, const JshLaunchShape& shape, unsigned int* queue,
                                      int num_sms, cudaStream_t stream) {
  if (schedule == JSH_SCHED_STATIC) {
    const int bs = 128;
    unsigned blocks = (unsigned)((max_items + bs - 1) / bs);
    if (full) transfer_static_mixed_kernel<true><<<blocks, bs, 0, stream>>>(d_reqs, n_req);
    else transfer_static_mixed_kernel<false><<<blocks, bs, 0, stream>>>(d_reqs, n_req);
    return cudaGetLastError();
  }
  int bs = shape.block_size;
  if (bs > 256) bs = 256;
  int per_sm = shape.ctas_per_sm > 0 ? shape.ctas_per_sm : jsh_persistent_occupancy(JSH_PREC_MIXED, full, bs);
  if (per_sm < 1) per_sm = 1;
  unsigned blocks = (unsigned)(num_sms * per_sm);
  uint64_t need = (max_items + 31) / 32 * 32;
  if ((uint64_t)blocks * bs > need) blocks = (unsigned)((need + bs - 1) / bs);
  if (blocks == 0) blocks = 1;
  unsigned long long* q = (unsigned long long*)queue;
  if (full) transfer_persistent_mixed_kernel<true><<<blocks, bs, 0, stream>>>(d_reqs, n_req, q, shape.refill_threshold);
  else transfer_persistent_mixed_kernel<false><<<blocks, bs, 0, stream>>>(d_reqs, n_req, q, shape.refill_threshold);
  return cudaGetLastError();
}

int jsh_queue64_occupancy(int block_size);

int jsh_persistent_occupancy(int precision, bool full, int block_size) {
  int n = 0;
  if (precision == JSH_PREC_MIXED) {
    if (full) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, transfer_persistent_mixed_kernel<true>, block_size, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, transfer_persistent_mixed_kernel<false>, block_size, 0);
  } else {
    n = jsh_queue64_occupancy(block_size);
  }
  return n;
}

// ------------------------------------------------------------------ host
// Per-request and per-frequency constants of the FP32 coefficient algebra,
// evaluated in FP64 from the compiled model.
int jsh_prepare_mixed(JshRequest* req, const double* nu_host, JshFreqConst* fc) {
  const JshModel& m = req->model;
  JshMixed& X = req->mix;
  const JshFreqConst* keep = X.fc;
  memset(&X, 0, sizeof(X));
  X.fc = keep;
  const double s = m.s;
  const double nx = -req->plane.dx, ny = -req->plane.dy, nz = -req->plane.dz;
  X.nl[0] = (float)nx;
  X.nl[1] = (float)ny;
  X.nl[2] = (float)nz;
  X.pk = (float)((s + 2.) / 2.);
  X.dt_max_pc = req->P.dt_max / JSH_PC;
  X.kq = (float)m.kq_ratio;
  X.eq = (float)m.eq_ratio;
  if (m.v_kind == JSH_V_CONST_FLAT) {
    // getG, getD, get_n_los_prime (src/utils.cpp:147-162) in FP64
    double g = m.vp[0];
    double v = JSH_C * sqrt(1. - 1. / (g * g));
    double beta = v / JSH_C;
    double gamma = sqrt(1. / (1. - beta * beta));
    double D = 1. / (gamma * (1. - beta * nz));
    double f = (D + 1.) * (gamma / (gamma + 1.));
    X.v_const = 1;
    X.D = (float)D;
    X.gamma = (float)gamma;
    X.beta = (float)beta;
    X.nlp[0] = (float)(D * nx);
    X.nlp[1] = (float)(D * ny);
    X.nlp[2] = (float)(D * nz - f * beta);
  }
  const double cb = JSH_Q_E / (2. * JSH_PI * JSH_M_E * JSH_C);  // nu_B per gauss
  const double cp = JSH_Q_E * JSH_Q_E / (JSH_PI * JSH_M_E);     // nu_p^2 per cm^-3
  const double fki = m.b_scalar ? m.fk_i * m.rnd_k : m.fk_i;
  const double fei = m.b_scalar ? m.fe_i * m.rnd_e : m.fe_i;
  for (int i = 0; i < req->n_nu; ++i) {
    double nu = nu_host[i];
    double Ak = JSH_PI * cp * pow(cb, (s + 2.) / 2.) * fki / (JSH_C * pow(nu, (s + 4.) / 2.));
    double Ae = JSH_PI * cp * pow(cb, (s + 1.) / 2.) * JSH_M_E * fei / (JSH_C * pow(nu, (s - 1.) / 2.));
    double Av = JSH_PI * cp * pow(cb, (s + 3.) / 2.) * m.fk_v / (JSH_C * pow(nu, (s + 5.) / 2.));
    double Aev = JSH_PI * cp * pow(cb, 1. + s / 2.) * JSH_M_E * m.fe_v / (JSH_C * pow(nu, s / 2.));
    double Af = 2. * JSH_PI * cp * cb / (JSH_C * nu * nu) * (m.kfr_factor + m.thermal_fraction);
    double Ac = JSH_PI * cp * cb * cb / (JSH_C * nu * nu * nu);
    double Gnu = pow(cb / nu, (s - 2.) / 2.);
    // scale: the source function at w = 1, D = 1
    double S = exp2(nearbyint(log2(Ae / Ak)));
    JshFreqConst& F = fc[i];
    F.ak = (float)(Ak * JSH_PC);
    F.ae = (float)(Ae * JSH_PC / S);
    F.av = (float)(Av * JSH_PC);
    F.aev = (float)(Aev * JSH_PC / S);
    F.af = (float)(Af * JSH_PC);
    F.ac = (float)(Ac * JSH_PC);
    F.c1 = (float)(m.kcr_a * m.kcr_b + m.thermal_fraction);
    F.c2 = (float)(m.kcr_a * Gnu);
    F.scale = S;
    F.atol = req->P.atol / S;
    const float vals[6] = {F.ak, F.ae, F.av, F.aev, F.af, F.ac};
    for (float x : vals) {
      if (!isfinite(x) || (x != 0.f && fabsf(x) < 1e-30f)) {
        jsh_set_error("frequency %g Hz puts the mixed-precision coefficients outside FP32 range; use FP64", nu);
        return JSH_ERR_INVALID;
      }
    }
  }
  return JSH_OK;
}
