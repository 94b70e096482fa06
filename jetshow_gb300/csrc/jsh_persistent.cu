// jsh_persistent.cu -- the mixed-precision transfer: FP32 right-hand sides
// and Runge-Kutta stages; FP64 time, step size, accumulated optical depth
// and Faraday rotation angle.  One work item is a (request, hit ray,
// frequency); its tau pass (src/Observation.cpp:126-214; a quadrature here,
// adaptive Gauss-Kronrod panels) and I/IQUV pass (src/Observation.cpp:242-308,
// src/System.cpp:41-63; Dormand-Prince) run as a per-lane state machine that
// advances by one panel or one Dormand-Prince attempt per call, so that
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
//
// Code size matters as much as arithmetic here: the stages run as a rolled
// loop over a __constant__ tableau with the stage derivatives in shared
// memory, so the coefficient code exists once per kernel and the kernel
// fits the SM instruction caches even when the lanes of a warp are in
// different phases.
#include <float.h>
#include <math.h>

#include <algorithm>
#include <mutex>
#include <unordered_map>

#include "jsh_batch.cuh"
#include "jsh_context.h"
#include "jsh_fields.cuh"
#include "jsh_fields32.cuh"
#include "jsh_launch.h"
#include "jsh_quadrature.h"
#include "jsh_transfer64.cuh"

namespace jsh {

namespace {

constexpr uint8_t PH_IDLE = 0, PH_TAU = 1, PH_IQUV = 2;
// Which passes a lane machine runs: both (the static schedule and the
// single-kernel persistent form), the tau pass only (the split form's first
// kernel: an item that needs an I/IQUV pass is handed on as a JshIquvItem),
// or the I/IQUV pass only (the split form's second kernel).
constexpr int PASS_BOTH = 0, PASS_TAU = 1, PASS_IQUV = 2;
// Optical depth of the equilibrium start of full-Stokes IQUV passes.
// Measured with the oracle's coefficients against the integration from
// tau_max (scipy Radau at rtol 1e-11) on 27 rays of depth 94 .. 3.2e4 of the
// conical and ParabaloidCone jets at their lowest and highest frequencies:
// worst 2.2e-6 of I in I, Q, U, V at tau_eq = 30 (2.6e-5 at 20), against
// 3e-10 for the zero state at tau_thick = 89.
constexpr double kTauEq = 30.0;
// Smallest total depth of a ray started in equilibrium at kTauEq: behind the
// start lie at least 10 optical depths, so the state there is within
// exp(-(1 - p) 10) of equilibrium before the 30 depths in front attenuate it.
// The rays just shallower than this, integrated whole from their far end,
// are the render's longest items (their cost grows with their depth): on the
// 512x1024 conical jet lowering it from 50 to 40 took the longest from 4 585
// to 3 883 evaluations with the errors against the converged oracle of 300
// rays of depth 25 .. 80 unchanged (I 5.8e-6, Q 4.1e-6 of max I; 35 raised
// Q to 6.8e-6).
constexpr double kTauEqMin = 40.0;
constexpr double INV_PC = 1.0 / JSH_PC;
// First panel width of a tau-pass segment: a quarter of it (the panels then
// adapt; four panels of 15 nodes resolve the features of a segment that one
// panel's error estimate could miss).
constexpr float kPanelsPerSegment = 4.f;

// Tableau entry a_sj in FP32 (row 6 = the 5th-order weights b), folded to an
// immediate operand where s and j are compile-time constants.
__host__ __device__ constexpr float dp_a32(int s, int j) {
  return s == 1 ? (j == 0 ? (float)dp::A21 : 0.f)
       : s == 2 ? (j == 0 ? (float)dp::A31 : j == 1 ? (float)dp::A32 : 0.f)
       : s == 3 ? (j == 0 ? (float)dp::A41 : j == 1 ? (float)dp::A42 : j == 2 ? (float)dp::A43 : 0.f)
       : s == 4 ? (j == 0 ? (float)dp::A51 : j == 1 ? (float)dp::A52 : j == 2 ? (float)dp::A53
                  : j == 3 ? (float)dp::A54 : 0.f)
       : s == 5 ? (j == 0 ? (float)dp::A61 : j == 1 ? (float)dp::A62 : j == 2 ? (float)dp::A63
                  : j == 3 ? (float)dp::A64 : j == 4 ? (float)dp::A65 : 0.f)
       : s == 6 ? (j == 0 ? (float)dp::B1 : j == 2 ? (float)dp::B3 : j == 3 ? (float)dp::B4
                  : j == 4 ? (float)dp::B5 : j == 5 ? (float)dp::B6 : 0.f)
       : 0.f;
}

// Dormand-Prince nodes c, error weights e = b - b_hat and dense-output
// weights d in FP32.
__constant__ float c_C[7] = {0, (float)dp::C2, (float)dp::C3, (float)dp::C4, (float)dp::C5, 1.f, 1.f};
__constant__ float c_E[7] = {(float)dp::E1, 0, (float)dp::E3, (float)dp::E4, (float)dp::E5, (float)dp::E6,
                             (float)dp::E7};
__constant__ float c_D[7] = {(float)dp::D1, 0, (float)dp::D3, (float)dp::D4, (float)dp::D5, (float)dp::D6,
                             (float)dp::D7};
// 5th-order weights b of the first six stages (b_7 = 0)
__constant__ float c_B[6] = {(float)dp::B1, 0, (float)dp::B3, (float)dp::B4, (float)dp::B5, (float)dp::B6};

// Compensated FP32 pair x = hi + lo, |lo| <= ulp(hi) / 2 (about 48 bits):
// the step-control state (segment coordinate, remainder, optical depth,
// Faraday angle, base point) is carried in these pairs because GB300 runs
// FP64 at 1/64 of the FP32 rate; the additions are error-free
// transformations (Knuth's two-sum, Dekker's product error by fma).
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_of(double x) {
  const float h = (float)x;
  return DF{h, (float)(x - (double)h)};
}
__device__ __forceinline__ double df_val(DF a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ DF df_norm(float s, float e) {
  const float hi = s + e;
  return DF{hi, e - (hi - s)};
}
// a + b
__device__ __forceinline__ DF df_add(DF a, float b) {
  const float s = a.hi + b;
  const float bb = s - a.hi;
  const float e = ((a.hi - (s - bb)) + (b - bb)) + a.lo;
  return df_norm(s, e);
}
// a - b
__device__ __forceinline__ DF df_sub(DF a, DF b) {
  const float s = a.hi - b.hi;
  const float bb = s - a.hi;
  const float e = ((a.hi - (s - bb)) - (b.hi + bb)) + (a.lo - b.lo);
  return df_norm(s, e);
}
// p + t * d rounded to FP32 (p, t, d pairs)
__device__ __forceinline__ float df_axpy_round(DF t, DF d, DF p) {
  const float m = t.hi * d.hi;
  const float me = fmaf(t.hi, d.hi, -m);  // exact product error
  const float s = p.hi + m;
  const float bb = s - p.hi;
  const float se = (p.hi - (s - bb)) + (m - bb);
  return s + (((se + me) + p.lo) + fmaf(t.hi, d.lo, t.lo * d.hi));
}

struct Lane {
  int r, f;
  uint32_t h;
  uint8_t phase;
  int8_t seg, nseg;
  int8_t first_seg;      // segment where the IQUV pass starts inside (-1: at its end)
  bool init;
  bool last;             // dt was truncated to reach the segment's end
  uint8_t ft;            // IQUV pass in the Faraday-thick mode (quasi-static polarisation)
  uint8_t ft_cool;       // steps before the Faraday-thick mode may be tried again
  uint8_t ft_back;       // entry estimates in a row that found the transient too large (back-off)
  DF p0x, p0y, p0z;      // segment start [pc]
  float bx, by, bz;      // p0 + t d rounded to FP32 after each accepted step:
                         // stage points are b + c h d in FP32 (error u |b|)
  DF length, t;          // segment length and coordinate [pc]
  float dt;              // [pc]
  double length_cm;
  DF tau_seg;            // optical depth of the current tau segment
  float thick_left;      // tau_thick - (depth of the finished segments)
  double tau_bg, thick;
  double t_first;        // [pc] IQUV start on first_seg: tau_max crossing or optically thick point
  DF chi;                // Faraday rotation angle, kept reduced to [-pi, pi]
  float x[4];
  float k1[5];
  float s1;  // noise scale of k1
  float kI1; // k_I at the point of k1
  int32_t nsteps, fails;
  uint32_t status;
  uint32_t evals, acc, rej;
  uint32_t evals0;       // split form, IQUV kernel: the item's tau-pass evaluations (cost map)
  int32_t tri;           // gridded fields on one grid: triangle of the last evaluation (-1: none)
};

// Stage derivatives of this thread, thread-major: t[s * NK + c] with t =
// shared + tid * W.  Every access is a compile-time offset from one base
// register (no per-access address arithmetic), and W = 35 or 7 floats maps
// a warp's 32 threads onto 32 distinct banks (W odd).  W is the per-thread
// region of the kernel's buffer, so a one-component view of a 5-component
// buffer (the single-kernel form's tau lanes) stays inside its own thread.
template <int NK, int W = 7 * NK>
struct Stages {
  float* t;
  __device__ __forceinline__ float& operator()(int s, int c) const { return t[s * NK + c]; }
};

// acc = sum_{j < S} a_Sj K_j with S and j compile-time: the tableau entries
// are immediate operands and the S*NK shared loads are independent.
template <int S, int NK, int W>
__device__ __forceinline__ void combine_stage(const Stages<NK, W>& K, float* acc) {
#pragma unroll
  for (int c = 0; c < NK; ++c) acc[c] = 0.f;
#pragma unroll
  for (int j = 0; j < S; ++j) {
#pragma unroll
    for (int c = 0; c < NK; ++c) acc[c] = fmaf(dp_a32(S, j), K(j, c), acc[c]);
  }
}

template <int NK, int W>
__device__ __forceinline__ void combine(int s, const Stages<NK, W>& K, float* acc) {
  switch (s) {
    case 1: combine_stage<1, NK, W>(K, acc); break;
    case 2: combine_stage<2, NK, W>(K, acc); break;
    case 3: combine_stage<3, NK, W>(K, acc); break;
    case 4: combine_stage<4, NK, W>(K, acc); break;
    case 5: combine_stage<5, NK, W>(K, acc); break;
    default: combine_stage<6, NK, W>(K, acc); break;
  }
}

__device__ __forceinline__ double seg_len_cm(const JshHit& H, int s, double ox, double oy, double oz) {
  double dx = ox - H.seg[s][0], dy = oy - H.seg[s][1], dz = oz - H.seg[s][2];
  return sqrt((dx * dx + dy * dy) + dz * dz);
}

// auto_n of src/Observation.cpp:254-258: steps_schedule (src/utils.cpp:354-366,
// default limits 0.1 and 100) in FP32.  It only sets the first step guess of
// a segment, so FP32 rounding near an integer boundary changes no accuracy;
// in FP64 its log and pow were a large share of the per-item FP64 work
// (GB300 runs FP64 at 1/64 of the FP32 rate).
__device__ __forceinline__ float first_step_divisor(double tau_bg, int n) {
  if (!(tau_bg > 0.1)) return (float)n;
  if (tau_bg >= 100.0) return (float)(10 * n);
  const float b = 2.30258509f;                              // -log(0.1)
  const float k = (float)(10 * n) / ((4.60517019f + b) * (4.60517019f + b));  // log(100) + b
  const float l = logf((float)tau_bg) + b;
  return ceilf(fmaf(k * l, l, (float)n));
}

__device__ __forceinline__ void set_segment(Lane& L, double ox, double oy, double oz, double length_cm) {
  L.length_cm = length_cm;
  const double len = length_cm * INV_PC;
  L.length = df_of(len);
  L.t = DF{0.f, 0.f};
  L.p0x = df_of(ox * INV_PC);
  L.p0y = df_of(oy * INV_PC);
  L.p0z = df_of(oz * INV_PC);
  L.bx = L.p0x.hi;
  L.by = L.p0y.hi;
  L.bz = L.p0z.hi;
  L.last = false;
  L.init = false;
  L.nsteps = 0;
  L.fails = 0;
}

__device__ __forceinline__ void begin_tau_segment(Lane& L, const JshRequest& R, const JshHit& H) {
  int s = L.seg;
  set_segment(L, H.seg[s][0], H.seg[s][1], H.seg[s][2], seg_len_cm(H, s, H.seg[s][3], H.seg[s][4], H.seg[s][5]));
  const float len = L.length.hi + L.length.lo;
  L.tau_seg = DF{0.f, 0.f};
  L.thick_left = (float)(R.mix.tau_eq - L.tau_bg);
  if (!R.mix.helical_log) {
    // the Dormand-Prince tau pass: the reference's first step L / n
    L.dt = len / (float)R.P.n;
    return;
  }
  L.dt = len * (1.f / kPanelsPerSegment);
  // closest approach of the segment to the jet (z) axis, where the fields'
  // azimuthal direction turns fastest (a helical B flips within the
  // approach distance): a panel breakpoint when it lies inside the segment
  // and the approach distance is below 1/32 of the segment, finer than the
  // nodes of the first panels resolve (L.k1[2], [pc] along it; L.k1[3] the
  // approach distance, at least 1e-6 of the segment).  FP32 is enough: it
  // only places panels.
  const float ux = R.mix.dhi[0], uy = R.mix.dhi[1];
  const float uu = fmaf(ux, ux, uy * uy);
  L.k1[2] = INFINITY;
  L.k1[3] = 1e-6f * len;
  if (uu > 0.f) {
    const float sc = -fmaf(L.p0x.hi, ux, L.p0y.hi * uy) / uu;
    if (sc > 0.f && sc < len) {
      const float cx = fmaf(sc, ux, L.p0x.hi), cy = fmaf(sc, uy, L.p0y.hi);
      const float rmin = sqrtf(fmaf(cx, cx, cy * cy));
      if (rmin < len * (1.f / 32.f)) {
        L.k1[2] = sc;
        L.k1[3] = fmaxf(rmin, L.k1[3]);
      }
    }
  }
}

__device__ __forceinline__ void begin_iquv_segment(Lane& L, const JshRequest& R, const JshHit& H) {
  int s = L.seg;
  double ox = H.seg[s][3], oy = H.seg[s][4], oz = H.seg[s][5];
  if (s == L.first_seg) {
    L.first_seg = -1;
    double tc = L.t_first * JSH_PC;
    ox = H.seg[s][0] + R.plane.rx * tc;
    oy = H.seg[s][1] + R.plane.ry * tc;
    oz = H.seg[s][2] + R.plane.rz * tc;
  }
  set_segment(L, ox, oy, oz, seg_len_cm(H, s, ox, oy, oz));
  L.dt = (L.length.hi + L.length.lo) / first_step_divisor(L.tau_bg, R.P.n);
  L.ft = 0;  // (Q, U) enters a segment as it left the last one, not quasi-static
  L.ft_cool = 0;
  L.ft_back = 0;
}

// Work item w of the batch.  Unranked: frequency-major over the hit list.
// Ranked (persistent schedule): all frequencies of a ray together, rays in
// the heaviest-first order of the ranking kernels; part 1 (the rays after
// the deep prefix of overlapped passes) starts after the deep prefix.
__device__ __forceinline__ void lane_start(Lane& L, const JshRequest* __restrict__ reqs,
                                           const unsigned long long* base, int n_req, unsigned long long w,
                                           bool ranked, int part = 0) {
  int r = find_request(base, n_req, w);
  const JshRequest& R = reqs[r];
  unsigned long long local = w - base[r];
  L.r = r;
  if (ranked) {
    const unsigned long long rank = local / (unsigned)R.n_nu;
    L.f = (int)(local - rank * (unsigned)R.n_nu);
    L.h = R.order[rank + (part ? R.buckets[JSH_RANK_DEEP] : 0u)];
  } else {
    unsigned nhit = *R.n_hit;
    L.f = (int)(local / nhit);
    L.h = (uint32_t)(local % nhit);
  }
  const JshHit& H = R.hits[L.h];
  L.phase = PH_TAU;
  L.seg = 0;
  L.nseg = (int8_t)H.nseg;
  L.first_seg = -1;
  L.tau_bg = 0.0;
  L.thick = 0.0;
  L.t_first = -1.0;
  L.chi = DF{0.f, 0.f};
  L.x[0] = L.x[1] = L.x[2] = L.x[3] = 0.f;
  L.status = (uint32_t)H.status | JSH_ST_HIT;
  L.evals = L.acc = L.rej = 0;
  L.tri = -1;
  L.ft = 0;
  L.ft_cool = 0;
  L.evals0 = 0;
  begin_tau_segment(L, R, H);
}

// Per-lane totals of a request's counters (right-hand-side evaluations,
// accepted and rejected steps, status OR) over the items the lane finished
// or handed on.  They reach the request's counters when the lane moves to an
// item of another request (per lane) and when the kernel ends (one atomic
// per warp and counter), instead of four atomics per item on the same four
// words: those kept one L2 slice's atomic unit busy for ~60 % of the tau
// kernel's time and set its length once its arithmetic shrank.
struct Tally {
  int r;
  unsigned long long evals;
  uint32_t acc, rej, status;
};

__device__ __forceinline__ Tally tally_new() { return Tally{-1, 0ull, 0u, 0u, 0u}; }

__device__ __forceinline__ void tally_add(Tally& T, const JshRequest* __restrict__ reqs, int r, uint32_t evals,
                                          uint32_t acc, uint32_t rej, uint32_t status) {
  if (r != T.r) {
    if (T.r >= 0) {
      unsigned long long* c = reqs[T.r].counters;
      atomicAdd(&c[0], T.evals);
      atomicAdd(&c[1], (unsigned long long)T.acc);
      atomicAdd(&c[2], (unsigned long long)T.rej);
      atomicOr(&c[3], (unsigned long long)T.status);
    }
    T = Tally{r, 0ull, 0u, 0u, 0u};
  }
  T.evals += evals;
  T.acc += acc;
  T.rej += rej;
  T.status |= status;
}

// Flush at the end of a kernel; every lane of the warp calls it.
__device__ __forceinline__ void tally_flush(const Tally& T, const JshRequest* __restrict__ reqs) {
  add_counters(reqs, T.r, T.r >= 0, T.evals, T.acc, T.rej, T.status);
}

// Writes one finished item (the Stokes vector rotated back to the lab frame
// in FP64); its counters go to the lane's tally.
__device__ __noinline__ void write_finished(const JshRequest* __restrict__ reqs, int r, int f, uint32_t h,
                                            double tau_bg, double thick, float chi_hi, float chi_lo, float x0,
                                            float x1, float x2, float x3, uint32_t status, uint32_t evals) {
  const JshRequest& R = reqs[r];
  const JshHit& H = R.hits[h];
  uint64_t q = (uint64_t)f * R.npix + (uint64_t)H.pix;
  double S = R.mix.fc[f].scale;
  // rotation by chi = hi + lo (|hi| <= pi): sin, cos of hi in FP32 and the
  // first-order correction for lo; (Q, U) need ~1e-7 of P, far above this
  float sh, ch;
  sincosf(chi_hi, &sh, &ch);
  const float ss = fmaf(chi_lo, ch, sh), sc = fmaf(-chi_lo, sh, ch);
  if (R.tau) R.tau[q] = tau_bg;
  if (R.l) R.l[q] = (R.P.flags & JSH_FLAG_COST_MAP) ? (double)evals : thick;
  if (R.I) R.I[q] = S * (double)x0;
  if (R.Q) R.Q[q] = S * (double)fmaf(sc, x1, -ss * x2);
  if (R.U) R.U[q] = S * (double)fmaf(ss, x1, sc * x2);
  if (R.V) R.V[q] = S * (double)x3;
  if (R.status) R.status[q] = status;
}

__device__ __forceinline__ void lane_finish(Lane& L, const JshRequest* __restrict__ reqs, Tally& T) {
  write_finished(reqs, L.r, L.f, L.h, L.tau_bg, L.thick, L.chi.hi, L.chi.lo, L.x[0], L.x[1], L.x[2], L.x[3],
                 L.status, L.evals);
  tally_add(T, reqs, L.r, L.evals, L.acc, L.rej, L.status);
  L.phase = PH_IDLE;
}

// Split form, IQUV kernel: the item's Stokes planes and final status (its
// tau and l planes were written by the tau kernel; with the cost map, l is
// rewritten with the evaluations of both passes).
__device__ __noinline__ void write_finished_iquv(const JshRequest* __restrict__ reqs, int r, int f, uint32_t h,
                                                 float chi_hi, float chi_lo, float x0, float x1, float x2,
                                                 float x3, uint32_t status, uint32_t evals0, uint32_t evals) {
  const JshRequest& R = reqs[r];
  const JshHit& H = R.hits[h];
  uint64_t q = (uint64_t)f * R.npix + (uint64_t)H.pix;
  double S = R.mix.fc[f].scale;
  float sh, ch;
  sincosf(chi_hi, &sh, &ch);
  const float ss = fmaf(chi_lo, ch, sh), sc = fmaf(-chi_lo, sh, ch);
  if (R.l && (R.P.flags & JSH_FLAG_COST_MAP)) R.l[q] = (double)(evals0 + evals);
  if (R.I) R.I[q] = S * (double)x0;
  if (R.Q) R.Q[q] = S * (double)fmaf(sc, x1, -ss * x2);
  if (R.U) R.U[q] = S * (double)fmaf(ss, x1, sc * x2);
  if (R.V) R.V[q] = S * (double)x3;
  if (R.status) R.status[q] = status;
}

// Optical depth the I/IQUV pass of an item integrates through (its cost
// grows with it), bucketed by half octaves; everything below 0.5 in bucket 1.
__device__ __forceinline__ uint8_t iquv_cost_key(double tau_bg, bool eq, bool first, const JshMixed& X) {
  double d = eq ? X.tau_eq : (first ? fmin(tau_bg, X.tau_thick) : tau_bg);
  if (!(d > 0.5)) return 1;
  const int k = (int)floorf(2.f * __log2f((float)d)) + 3;
  return (uint8_t)min(max(k, 1), JSH_RANK_BUCKETS - 1);
}

// Split form, tau kernel: hand an item whose I/IQUV pass is still to run to
// the IQUV kernel.  Writes the item's tau and l planes and its tau-pass
// counters, appends its record to the request's list of its part (one
// atomic per request among the lanes that emit together).
__device__ __noinline__ void emit_iquv(const JshRequest* __restrict__ reqs, int part, int r, int f, uint32_t h,
                                       double tau_bg,
                                       double thick, double t_first, int first_seg, int nseg, bool eq,
                                       uint32_t status, uint32_t evals) {
  const JshRequest& R = reqs[r];
  const JshHit& H = R.hits[h];
  uint64_t q = (uint64_t)f * R.npix + (uint64_t)H.pix;
  if (R.tau) R.tau[q] = tau_bg;
  if (R.l) R.l[q] = (R.P.flags & JSH_FLAG_COST_MAP) ? (double)evals : thick;
  const unsigned mask = __activemask();
  const unsigned peers = __match_any_sync(mask, r);
  const int leader = __ffs(peers) - 1;
  const unsigned lane = threadIdx.x & 31u;
  uint32_t slot = 0;
  if ((int)lane == leader) slot = atomicAdd(R.iq_count + part, (uint32_t)__popc(peers));
  slot = __shfl_sync(peers, slot, leader) + (uint32_t)__popc(peers & ((1u << lane) - 1u));
  if (part) slot += R.buckets[JSH_RANK_DEEP] * (uint32_t)R.n_nu;
  JshIquvItem it;
  it.h = h;
  it.f = (uint16_t)f;
  it.key = iquv_cost_key(tau_bg, eq, first_seg >= 0, R.mix);
  it.flags = (uint8_t)((nseg & 3) | (eq ? 4 : 0) | ((first_seg + 1) << 3));
  it.status = status;
  it.evals = evals;
  it.tau_bg = tau_bg;
  it.t_first = t_first;
  R.iq_items[slot] = it;
}

// Bisection for the tau_max crossing on the dense output of the last
// Dormand-Prince step (src/Observation.cpp:166-190); returns the crossing
// time [pc], or -1 without convergence.
__device__ __noinline__ double crossing_time(double tau_old, double t_old, double dt_used, float h, float k1,
                                             float k3, float k4, float k5, float k6, float k7, float inc,
                                             double tau_max, double tau_prec) {
  const float ydiff = inc;
  const float bspl = h * k1 - ydiff;
  const float r4 = ydiff - h * k7 - bspl;
  const float r5 = h * (c_D[0] * k1 + c_D[2] * k3 + c_D[3] * k4 + c_D[4] * k5 + c_D[5] * k6 + c_D[6] * k7);
  double t0 = t_old, t1 = t_old + dt_used, xm = tau_old + (double)inc, tm;
  int it = 0;
  while (fabs(xm - tau_max) > tau_prec) {
    if (++it > 200) return -1.0;
    tm = 0.5 * (t0 + t1);
    float th = (float)((tm - t_old) / dt_used), th1 = 1.f - th;
    xm = tau_old + (double)(th * (ydiff + th1 * (bspl + th * (r4 + th1 * r5))));
    if (xm > tau_max) t1 = tm;
    else t0 = tm;
  }
  return 0.5 * (t0 + t1);
}

// Coefficients and Stokes derivatives of the I/IQUV pass (one call site per
// kernel); `full` = false stops after k_I, eta_I (I-only output).  Returns
// the magnitude of the terms summed into the derivatives (eta_I + k_I |I|):
// the scale of their FP32 rounding noise.
template <bool GENERAL>
__device__ __forceinline__ float rhs32(const JshRequest& R, const JshFreqConst& F, bool full, F3 p, const float* y,
                                       float cs, float sn, float* dk, float& kI, uint32_t rk_h, uint32_t rk_f,
                                       uint32_t rk_e, int* tri, bool ft = false, float* cpl = nullptr) {
  Coef32 c;
  coef32_rt<GENERAL>(R, F, p, full ? COEF_FULL : COEF_I, c, rk_h, rk_f, rk_e, tri);
  kI = c.kI;
  const float scale = fabsf(c.eI) + fabsf(c.kI * y[0]);
  if (!full) {
    dk[0] = c.eI - c.kI * y[0];
    dk[1] = dk[2] = dk[3] = dk[4] = 0.f;
    return scale;
  }
  if (ft) {
    // Faraday-thick mode: the lab-frame polarisation Pi = Q + iU obeys
    // Pi' = -lambda Pi + S, lambda = k_I - i k_F, S = (eta_Q - k_Q I) - i k_C V.
    // Where |lambda| is far above the rate at which S / lambda changes, Pi is
    // that quasi-static value plus a transient d whose rotating-frame value
    // only decays (d' = -k_I d, up to the adiabatic lag); I and V see the
    // quasi-static part through k_Q Re Pi and k_C Im Pi, the transient's
    // share rotates at k_F and integrates to at most ~cpl |d|.  dk[1], dk[2]
    // carry the rotating-frame value e^{-i chi} S / lambda itself.
    const float sre = c.eQ - c.kQ * y[0], sim = -c.kC * y[3];
    const float il = 1.f / fmaf(c.kI, c.kI, c.kF * c.kF);
    const float pre = fmaf(sre, c.kI, -sim * c.kF) * il, pim = fmaf(sre, c.kF, sim * c.kI) * il;
    dk[0] = c.eI - c.kI * y[0] - c.kQ * pre - c.kV * y[3];
    dk[1] = fmaf(cs, pre, sn * pim);
    dk[2] = fmaf(-sn, pre, cs * pim);
    dk[3] = c.eV - c.kI * y[3] - c.kV * y[0] + c.kC * pim;
    dk[4] = c.kF;
    *cpl = fmaxf(fabsf(c.kQ), fabsf(c.kC)) * sqrtf(il);
    return scale;
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
  return scale;
}

// Local equilibrium of the transfer equation dx/dt = eps - K x at the IQUV
// start point of an optically thick ray (the end of the tau step that landed
// on tau_eq): x = K^-1 eps with the lab-frame transfer matrix of the
// reference's full-Stokes system (src/System.cpp:41-63; k_U = eta_U = h_Q = 0
// in its frame)
//     K = [[k_I, k_Q, 0, k_V], [k_Q, k_I, k_F, 0], [0, -k_F, k_I, k_C],
//          [k_V, 0, -k_C, k_I]],  eps = (eta_I, eta_Q, 0, eta_V),
// solved in FP64 by Gaussian elimination (K's symmetric part is positive
// definite: |k_Q|, |k_V| < k_I).  chi = 0 there, so the rotating frame is the
// lab frame.  The state is in the request's scaled intensity units, like the
// coefficients.  (ox, oy, oz): the start point [cm].
__device__ __noinline__ float4 equilibrium_state(const JshRequest* __restrict__ reqs, int r, int f, double ox,
                                                double oy, double oz) {
  const JshRequest& R = reqs[r];
  Coef32 c;
  coef32_rt(R, R.mix.fc[f], f3((float)(ox * INV_PC), (float)(oy * INV_PC), (float)(oz * INV_PC)), COEF_FULL, c);
  double A[4][5] = {{c.kI, c.kQ, 0.0, c.kV, c.eI},
                    {c.kQ, c.kI, c.kF, 0.0, c.eQ},
                    {0.0, -c.kF, c.kI, c.kC, 0.0},
                    {c.kV, 0.0, -c.kC, c.kI, c.eV}};
  // no pivoting: every leading block of K has a positive definite symmetric
  // part, so its pivots are nonzero
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (!(A[k][k] != 0.0)) return make_float4(0.f, 0.f, 0.f, 0.f);  // k_I = 0 there: zero state
#pragma unroll
    for (int i = k + 1; i < 4; ++i) {
      const double m = A[i][k] / A[k][k];
#pragma unroll
      for (int j = k; j < 5; ++j) A[i][j] -= m * A[k][j];
    }
  }
  double x[4];
#pragma unroll
  for (int i = 3; i >= 0; --i) {
    double a = A[i][4];
#pragma unroll
    for (int j = i + 1; j < 4; ++j) a -= A[i][j] * x[j];
    x[i] = a / A[i][i];
  }
  return make_float4((float)x[0], (float)x[1], (float)x[2], (float)x[3]);
}

__device__ __forceinline__ void lane_finish_iquv(Lane& L, const JshRequest* __restrict__ reqs, Tally& T) {
  write_finished_iquv(reqs, L.r, L.f, L.h, L.chi.hi, L.chi.lo, L.x[0], L.x[1], L.x[2], L.x[3], L.status, L.evals0,
                      L.evals);
  tally_add(T, reqs, L.r, L.evals, L.acc, L.rej, L.status);
  L.phase = PH_IDLE;
}

// First item slot of part `part`'s emitted items in iq_items / iq_order.
__device__ __forceinline__ uint32_t iq_first(const JshRequest& R, int part) {
  return part ? R.buckets[JSH_RANK_DEEP] * (uint32_t)R.n_nu : 0u;
}

// Split form, IQUV kernel: start work item w (heaviest-first over the
// batch's emitted items) where the tau kernel left it -- the I/IQUV pass's
// first segment, start point and state (zero, or the local equilibrium).
__device__ __forceinline__ void lane_start_iquv(Lane& L, const JshRequest* __restrict__ reqs,
                                                const unsigned long long* base, int n_req, unsigned long long w,
                                                int part) {
  const int r = find_request(base, n_req, w);
  const JshRequest& R = reqs[r];
  const JshIquvItem it = R.iq_items[R.iq_order[iq_first(R, part) + (uint32_t)(w - base[r])]];
  L.r = r;
  L.f = it.f;
  L.h = it.h;
  L.phase = PH_IQUV;
  L.nseg = (int8_t)(it.flags & 3);
  L.first_seg = (int8_t)((it.flags >> 3) & 3) - 1;
  const bool eq = (it.flags & 4) != 0;
  L.tau_bg = it.tau_bg;
  L.thick = 0.0;
  L.t_first = it.t_first;
  L.chi = DF{0.f, 0.f};
  L.x[0] = L.x[1] = L.x[2] = L.x[3] = 0.f;
  L.status = it.status;
  L.evals0 = it.evals;
  L.evals = L.acc = L.rej = 0;
  L.tri = -1;
  L.ft = 0;
  L.ft_cool = 0;
  L.seg = L.first_seg >= 0 ? L.first_seg : L.nseg - 1;
  const JshHit& H = R.hits[L.h];
  if (eq) {
    const int s = L.seg;
    const double tc = L.t_first * JSH_PC;
    const float4 xe = equilibrium_state(reqs, L.r, L.f, H.seg[s][0] + R.plane.rx * tc, H.seg[s][1] + R.plane.ry * tc,
                                        H.seg[s][2] + R.plane.rz * tc);
    L.x[0] = xe.x;
    L.x[1] = xe.y;
    L.x[2] = xe.z;
    L.x[3] = xe.w;
  }
  begin_iquv_segment(L, R, H);
}

// FP32 unit roundoff; the Stokes error norm's noise floor is
// kNoise * h * scale.  The rounding noise of the embedded error estimate of
// a Stokes component is about 0.3 u h scale (four terms of magnitude
// <= scale per derivative, weighted by |e_j| <= 0.05).
constexpr float kNoise = 5.9604645e-8f;
// This file is compiled twice: as is, and by jsh_persistent_ft.cu with
// JSH_FARADAY_THICK_BUILD 1 for requests that ask for the Faraday-thick mode
// (JSH_FLAG_FARADAY_THICK).  The mode's bookkeeping in the step costs the
// other requests ~18 % of the IQUV kernel even where it never engages, so
// the default kernels are built without it.
#ifndef JSH_FARADAY_THICK_BUILD
#define JSH_FARADAY_THICK_BUILD 0
#endif
constexpr bool kFtm = JSH_FARADAY_THICK_BUILD != 0;
// Faraday-thick mode of the IQUV pass: entry where
// |k_F| >= kFtRatio k_I; the quasi-static part's lag and the transient's
// left-out coupling must stay within kFtTol (atol + rtol I); after a refused
// entry or an exit the mode waits kFtCooldown accepted steps, after an entry
// estimate that found the transient too large kFtRetry, doubled for each
// such estimate in a row (up to 255).
constexpr float kFtRatio = 100.f;
constexpr float kFtTol = 1.f;
constexpr uint8_t kFtCooldown = 32;
constexpr int kFtRetry = 16;  // accepted steps after an entry estimate that found the transient too large
constexpr float kFtAxis = 0.25f;  // largest step / distance from the jet axis
// The mode's tolerance scales with I, as the full mode's own control of
// (Q, U) does through its noise floor (the quasi-static |Q + iU| is ~k_I/k_F
// of I where the mode applies).
__device__ __forceinline__ float ft_tolerance(float I, float rtol, float atol) {
  return kFtTol * fmaf(rtol, fabsf(I), atol);
}

// Stage components of the I/IQUV pass's Dormand-Prince machine: the IQUV
// state and chi (full Stokes) or I only.
template <bool FULL>
struct StageWidth {
  static constexpr int NK = FULL ? 5 : 1;
  static constexpr int NX = FULL ? 4 : 1;
};

// ---------------------------------------------------------------- tau pass
// The tau pass integrates dtau/dt = k_I along each segment.  Its right-hand
// side does not depend on the state, so the pass is a quadrature: each step
// is a Gauss-Kronrod 7/15 panel (jsh_quadrature.h) of adaptive width, with
// the adaptive-range semantics of the reference's Dormand-Prince pass
// (src/Observation.cpp:150-211: steps end exactly at the segment's end,
// dt_max bounds them, tau_max is located by bisection) and its tolerances
// (tau_atol, tau_rtol of the running segment depth).  A panel of 15 k_I
// evaluations replaces a step of 6: on the conical jet a tau pass needs
// ~2.3x fewer evaluations (an FP64 experiment on 600 C1 items: 75-97 per
// item against 195, errors 1e-9 .. 1e-12 of the converged depth).
__constant__ float c_gk_t[15] = {
    (float)(0.5 * (1.0 + jsh_gk15_x[0])),  (float)(0.5 * (1.0 + jsh_gk15_x[1])),
    (float)(0.5 * (1.0 + jsh_gk15_x[2])),  (float)(0.5 * (1.0 + jsh_gk15_x[3])),
    (float)(0.5 * (1.0 + jsh_gk15_x[4])),  (float)(0.5 * (1.0 + jsh_gk15_x[5])),
    (float)(0.5 * (1.0 + jsh_gk15_x[6])),  (float)(0.5 * (1.0 + jsh_gk15_x[7])),
    (float)(0.5 * (1.0 + jsh_gk15_x[8])),  (float)(0.5 * (1.0 + jsh_gk15_x[9])),
    (float)(0.5 * (1.0 + jsh_gk15_x[10])), (float)(0.5 * (1.0 + jsh_gk15_x[11])),
    (float)(0.5 * (1.0 + jsh_gk15_x[12])), (float)(0.5 * (1.0 + jsh_gk15_x[13])),
    (float)(0.5 * (1.0 + jsh_gk15_x[14]))};
__constant__ float c_gk_wk[15] = {
    (float)(0.5 * jsh_gk15_wk[0]),  (float)(0.5 * jsh_gk15_wk[1]),  (float)(0.5 * jsh_gk15_wk[2]),
    (float)(0.5 * jsh_gk15_wk[3]),  (float)(0.5 * jsh_gk15_wk[4]),  (float)(0.5 * jsh_gk15_wk[5]),
    (float)(0.5 * jsh_gk15_wk[6]),  (float)(0.5 * jsh_gk15_wk[7]),  (float)(0.5 * jsh_gk15_wk[8]),
    (float)(0.5 * jsh_gk15_wk[9]),  (float)(0.5 * jsh_gk15_wk[10]), (float)(0.5 * jsh_gk15_wk[11]),
    (float)(0.5 * jsh_gk15_wk[12]), (float)(0.5 * jsh_gk15_wk[13]), (float)(0.5 * jsh_gk15_wk[14])};
__constant__ float c_gk_wg[15] = {
    (float)(0.5 * jsh_gk15_wg[0]),  (float)(0.5 * jsh_gk15_wg[1]),  (float)(0.5 * jsh_gk15_wg[2]),
    (float)(0.5 * jsh_gk15_wg[3]),  (float)(0.5 * jsh_gk15_wg[4]),  (float)(0.5 * jsh_gk15_wg[5]),
    (float)(0.5 * jsh_gk15_wg[6]),  (float)(0.5 * jsh_gk15_wg[7]),  (float)(0.5 * jsh_gk15_wg[8]),
    (float)(0.5 * jsh_gk15_wg[9]),  (float)(0.5 * jsh_gk15_wg[10]), (float)(0.5 * jsh_gk15_wg[11]),
    (float)(0.5 * jsh_gk15_wg[12]), (float)(0.5 * jsh_gk15_wg[13]), (float)(0.5 * jsh_gk15_wg[14])};
__constant__ float c_gk_wd[15] = {
    (float)(0.5 * (jsh_gk15_wk[0] - jsh_gk15_wg[0])),   (float)(0.5 * (jsh_gk15_wg[1] - jsh_gk15_wk[1])),
    (float)(0.5 * (jsh_gk15_wk[2] - jsh_gk15_wg[2])),   (float)(0.5 * (jsh_gk15_wg[3] - jsh_gk15_wk[3])),
    (float)(0.5 * (jsh_gk15_wk[4] - jsh_gk15_wg[4])),   (float)(0.5 * (jsh_gk15_wg[5] - jsh_gk15_wk[5])),
    (float)(0.5 * (jsh_gk15_wk[6] - jsh_gk15_wg[6])),   (float)(0.5 * (jsh_gk15_wg[7] - jsh_gk15_wk[7])),
    (float)(0.5 * (jsh_gk15_wk[8] - jsh_gk15_wg[8])),   (float)(0.5 * (jsh_gk15_wg[9] - jsh_gk15_wk[9])),
    (float)(0.5 * (jsh_gk15_wk[10] - jsh_gk15_wg[10])), (float)(0.5 * (jsh_gk15_wg[11] - jsh_gk15_wk[11])),
    (float)(0.5 * (jsh_gk15_wk[12] - jsh_gk15_wg[12])), (float)(0.5 * (jsh_gk15_wg[13] - jsh_gk15_wk[13])),
    (float)(0.5 * (jsh_gk15_wk[14] - jsh_gk15_wg[14]))};
// Floor of a panel's tolerance on its error estimate K - G = h sum (w_K -
// w_G)_i k_i: each FP32 k_i carries a relative rounding error of up to
// ~2.6e-6 (exp2 of arguments up to ~60 in the log-domain coefficient form),
// so |K - G| is never resolved below 2.6e-6 h sum |w_K - w_G|_i |k_i|.  The
// floor is ~10x that: |K - G| bounds the Gauss rule's error, the Kronrod
// value kept is far more accurate, and panel widths grow only as the 15th
// root of the tolerance (on the 512x1024 conical jet 3x the noise bound and
// this floor gave 130 and 124 evaluations per tau pass, both with the
// worst tau 1.7e-6 off the converged oracle).
constexpr float kPanelNoise = 3e-5f;
// Bisection limit of the tau_max crossing inside a panel.
constexpr int kCrossIters = 48;

// The end of an item's tau pass: finish it (tau <= tau_min), hand it to the
// IQUV kernel (PASS_TAU) or start its I/IQUV pass in the same lane.
template <int PASS>
__device__ __forceinline__ void tau_pass_done(Lane& L, const JshRequest* __restrict__ reqs, int part, Tally& T) {
  const JshRequest& R = reqs[L.r];
  if (!(L.tau_bg > R.P.tau_min)) {
    lane_finish(L, reqs, T);
    return;
  }
  L.status |= JSH_ST_IQUV;
  L.phase = PH_IQUV;
  bool eq = false;
  if (L.first_seg >= 0 && R.mix.eq_start) {
    // the equilibrium start needs depth behind tau_eq: rays shallower than
    // eq_min are integrated whole from their far end
    if (L.tau_bg >= R.mix.eq_min || (L.status & JSH_ST_TAU_CROSSED)) eq = true;
    else L.first_seg = -1;
  }
  if (PASS == PASS_TAU) {
    emit_iquv(reqs, part, L.r, L.f, L.h, L.tau_bg, L.thick, L.t_first, L.first_seg, L.nseg, eq, L.status, L.evals);
    tally_add(T, reqs, L.r, L.evals, L.acc, L.rej, 0u);
    L.phase = PH_IDLE;
    return;
  }
  L.seg = L.first_seg >= 0 ? L.first_seg : L.nseg - 1;
  L.tri = -1;  // as the IQUV kernel's fresh lanes
  L.ft = 0;
  L.ft_cool = 0;
  const JshHit& H = R.hits[L.h];
  if (eq) {
    const int s = L.seg;
    const double tc = L.t_first * JSH_PC;
    const float4 xe = equilibrium_state(reqs, L.r, L.f, H.seg[s][0] + R.plane.rx * tc, H.seg[s][1] + R.plane.ry * tc,
                                        H.seg[s][2] + R.plane.rz * tc);
    L.x[0] = xe.x;
    L.x[1] = xe.y;
    L.x[2] = xe.z;
    L.x[3] = xe.w;
  }
  begin_iquv_segment(L, R, H);
}

// One panel of an active lane's tau pass (or a segment / pass transition).
// While the lane bisects a tau_max crossing (L.init set; the tau pass has
// no other use for it), the panel [t, t + w] with w the midpoint of the
// bracket [k1[0], k1[1]] is evaluated instead.
template <int PASS, bool GENERAL>
__device__ __forceinline__ void tau_panel_step(Lane& L, const JshRequest* __restrict__ reqs, int part, Tally& T) {
  const JshRequest& R = reqs[L.r];
  const JshFreqConst F = R.mix.fc[L.f];
  const bool bis = L.init;
  // integration direction: +d (away from the observer)
  const F3 dir = f3(-R.mix.nl[0], -R.mix.nl[1], -R.mix.nl[2]);
  bool at_bp = false;
  if (!bis) {
    const DF rem = df_sub(L.length, L.t);
    const float remf = rem.hi + rem.lo;
    if (!(remf > 0.f)) goto segment_done;
    if (R.mix.dt_max_f != 0.f && L.dt > R.mix.dt_max_f) L.dt = R.mix.dt_max_f;
    if (L.k1[2] < INFINITY) {
      // the segment's closest approach to the jet axis lies ahead: panels
      // close in on it by factors of 4 down to the approach distance and
      // end on it
      const DF rb = df_sub(DF{L.k1[2], 0.f}, L.t);
      const float rbf = rb.hi + rb.lo;
      if (rbf > 0.f) {
        L.dt = fminf(L.dt, fmaxf(0.75f * rbf, L.k1[3]));
        if (!(L.dt < rbf)) {
          L.dt = rbf;
          at_bp = true;
        }
      } else {
        L.k1[2] = INFINITY;
      }
    }
    L.last = !(L.dt < remf);
    if (L.last) {
      L.dt = remf;
      at_bp = false;
    }
  }
  if (L.nsteps++ >= R.P.max_steps) {
    L.status |= JSH_ST_STEP_LIMIT;
    goto abort;
  }
  {
    const float h = bis ? 0.5f * (L.k1[0] + L.k1[1]) : L.dt;
    const F3 pn = f3(L.bx, L.by, L.bz);
    float K = 0.f, G = 0.f, A = 0.f;
#pragma unroll 1
    for (int i = 0; i < 15; ++i) {
      Coef32 c;
      coef32_rt<GENERAL>(R, F, pn + dir * (c_gk_t[i] * h), COEF_KI, c, L.h, (uint32_t)L.f, L.evals + (uint32_t)i);
      K = fmaf(c_gk_wk[i], c.kI, K);
      G = fmaf(c_gk_wg[i], c.kI, G);
      A = fmaf(c_gk_wd[i], fabsf(c.kI), A);
    }
    L.evals += 15;
    K *= h;
    G *= h;
    if (!(K == K) || isinf(K)) {
      L.status |= JSH_ST_NAN;
      goto abort;
    }
    if (bis) {
      // tau at t + h against tau_max; stop within tau_precision of it
      // (src/Observation.cpp:166-185).  The crossing point starts the
      // I/IQUV pass; tau keeps the crossing panel's end value, as the
      // reference keeps the crossing step's (src/Observation.cpp:208).
      L.rej++;
      const double dv = df_val(df_add(L.tau_seg, K)) - R.P.tau_max;
      const bool done = fabs(dv) <= R.P.tau_precision || !(L.k1[1] - L.k1[0] > 1e-7f * L.k1[1]);
      if (!done && ++L.fails < kCrossIters) {
        if (dv > 0.0) L.k1[1] = h;
        else L.k1[0] = h;
        return;
      }
      if (!done) L.status |= JSH_ST_BISECT_LIMIT;
      L.init = false;
      L.tau_seg = DF{L.k1[2], L.k1[3]};
      L.first_seg = L.seg;
      L.t_first = df_val(L.t) + (double)h;
      L.nseg = L.seg + 1;
      L.tau_bg += df_val(L.tau_seg);
      L.thick += L.length_cm;
      tau_pass_done<PASS>(L, reqs, part, T);
      return;
    }
    // error test: |K - G| against the tolerance of the running depth, never
    // below the FP32 noise floor of the estimate
    const float err = fabsf(K - G);
    const float tol = fmaf(R.mix.tau_rtol, fabsf(L.tau_seg.hi) + fabsf(K), R.mix.tau_atol) + kPanelNoise * h * A;
    const float r = err > 0.f ? tol / err : 1e30f;
    if (!(r >= 1.f)) {
      L.dt = h * fminf(fmaxf(0.9f * __powf(r, 1.0f / 15.0f), 0.2f), 0.9f);
      L.last = false;
      L.rej++;
      if (++L.fails >= dp::FAIL_LIMIT) {
        L.status |= JSH_ST_FAIL_LIMIT;
        goto abort;
      }
      return;
    }
    // landing on the optically thick depth: a panel may not overshoot
    // tau_thick by more than 25 %, so that the IQUV pass can start at the end
    // of the crossing panel, where tau is as accurate as the integration
    if (L.first_seg < 0 && L.tau_seg.hi < L.thick_left && L.tau_seg.hi + K > 1.25f * L.thick_left) {
      L.dt = h * fmaxf((1.1f * L.thick_left - L.tau_seg.hi) / K, 0.01f);
      L.last = false;
      L.rej++;
      if (++L.fails >= dp::FAIL_LIMIT) {
        L.status |= JSH_ST_FAIL_LIMIT;
        goto abort;
      }
      return;
    }
    // tau_max inside this panel (the pass ends here): a crossing panel may
    // not overshoot tau_max by more than 25 % either (tau keeps its end
    // value); when no optically thick start precedes the crossing, the I/IQUV
    // pass starts at the crossing point, bisected for inside the panel
    {
      const DF tn = df_add(L.tau_seg, K);
      if (tn.hi > R.mix.tau_max_hi || (tn.hi == R.mix.tau_max_hi && tn.lo >= R.mix.tau_max_lo)) {
        if (tn.hi > 1.25f * R.mix.tau_max_hi) {
          L.dt = h * fmaxf((1.1f * R.mix.tau_max_hi - L.tau_seg.hi) / K, 0.01f);
          L.last = false;
          L.rej++;
          if (++L.fails >= dp::FAIL_LIMIT) {
            L.status |= JSH_ST_FAIL_LIMIT;
            goto abort;
          }
          return;
        }
        L.status |= JSH_ST_TAU_CROSSED;
        L.acc++;
        if (L.first_seg < 0) {
          L.init = true;
          L.k1[0] = 0.f;
          L.k1[1] = h;
          L.k1[2] = tn.hi;
          L.k1[3] = tn.lo;
          L.fails = 0;
          return;
        }
        L.tau_seg = tn;
        L.nseg = L.seg + 1;
        L.tau_bg += df_val(L.tau_seg);
        L.thick += L.length_cm;
        tau_pass_done<PASS>(L, reqs, part, T);
        return;
      }
    }
    // accept
    const DF t_prev = L.t;
    const DF t_new = L.last ? L.length : df_add(L.t, h);
    if (t_new.hi == t_prev.hi && t_new.lo == t_prev.lo) {
      L.status |= JSH_ST_DT_UNDERFLOW;
      goto abort;
    }
    L.t = t_new;
    L.bx = df_axpy_round(t_new, DF{R.mix.dhi[0], R.mix.dlo[0]}, L.p0x);
    L.by = df_axpy_round(t_new, DF{R.mix.dhi[1], R.mix.dlo[1]}, L.p0y);
    L.bz = df_axpy_round(t_new, DF{R.mix.dhi[2], R.mix.dlo[2]}, L.p0z);
    L.fails = 0;
    L.acc++;
    L.dt = h * fminf(fmaxf(0.9f * __powf(fminf(r, 1e15f), 1.0f / 15.0f), 1.f), 4.f);
    if (at_bp) {
      // past the closest approach: start again at the approach distance
      L.k1[2] = INFINITY;
      L.dt = L.k1[3];
    }
    L.tau_seg = df_add(L.tau_seg, K);
    if (L.first_seg < 0 && L.tau_seg.hi >= L.thick_left) {
      // optically thick from here on (tau within [1, 1.25] tau_thick): the
      // IQUV pass starts at the end of this panel; the tau pass goes on for
      // the tau image
      L.first_seg = L.seg;
      L.t_first = df_val(t_new);
    }
    return;
  }

segment_done : {
  L.tau_bg += df_val(L.tau_seg);
  L.thick += L.length_cm;
  if (L.seg + 1 < L.nseg) {
    L.seg++;
    begin_tau_segment(L, R, R.hits[L.h]);
    return;
  }
  tau_pass_done<PASS>(L, reqs, part, T);
  return;
}

abort:
  L.init = false;
  L.tau_bg += df_val(L.tau_seg);
  L.thick += L.length_cm;
  lane_finish(L, reqs, T);
}

// One Dormand-Prince attempt of an active lane's tau pass (the reference's
// stepper, src/Observation.cpp:150-211), for the requests whose fields may
// jump (sheaths, composite laws, cells, random and gridded fields: a
// quadrature panel's error estimate can miss a jump between its nodes).
// dtau/dt = k_I does not depend on the state, so only the last stage
// combination (the increment) is formed.
template <int PASS, bool GENERAL, int W>
__device__ __forceinline__ void tau_dopri_step(Lane& L, const JshRequest* __restrict__ reqs, const Stages<1, W>& K,
                                               int part, Tally& T) {
  const JshRequest& R = reqs[L.r];
  const JshFreqConst F = R.mix.fc[L.f];
  const F3 dirf = f3(-R.mix.nl[0], -R.mix.nl[1], -R.mix.nl[2]);
  const float max_dt = R.mix.dt_max_f;
  const float atol = R.mix.tau_atol;
  const float rtol = R.mix.tau_rtol;
  {
    const DF rem = df_sub(L.length, L.t);
    const float remf = rem.hi + rem.lo;
    if (!(remf > 0.f)) goto segment_done;
    L.last = !(L.dt < remf);
    if (L.last) L.dt = remf;
  }
  if (L.nsteps++ >= R.P.max_steps) {
    L.status |= JSH_ST_STEP_LIMIT;
    goto abort;
  }
  if (max_dt != 0.f && fabsf(L.dt) > max_dt) {
    L.dt = max_dt;
    L.rej++;
    if (++L.fails >= dp::FAIL_LIMIT) {
      L.status |= JSH_ST_FAIL_LIMIT;
      goto abort;
    }
    return;
  }
  {
    const F3 pn = f3(L.bx, L.by, L.bz);
    const float h = L.dt;
    if (!L.init) {
      Coef32 c;
      coef32_rt<GENERAL>(R, F, pn, COEF_KI, c, L.h, (uint32_t)L.f, L.evals, &L.tri);
      L.k1[0] = c.kI;
      L.evals++;
      L.init = true;
    }
    K(0, 0) = L.k1[0];
    float inc = 0.f;
#pragma unroll 1
    for (int s = 1; s < 7; ++s) {
      if (s == 6) {
        float acc[1];
        combine<1, W>(6, K, acc);
        inc = h * acc[0];
      }
      Coef32 c;
      coef32_rt<GENERAL>(R, F, pn + dirf * (c_C[s] * h), COEF_KI, c, L.h, (uint32_t)L.f,
                         L.evals + (uint32_t)(s - 1), &L.tri);
      K(s, 0) = c.kI;
    }
    L.evals += 6;
    float a = 0.f;
#pragma unroll
    for (int j = 0; j < 7; ++j) a = fmaf(c_E[j], K(j, 0), a);
    const float adt = fabsf(h);
    // no cancellation in dtau/dt = k_I: the plain odeint norm
    const float e = fabsf(h * a) / fmaf(rtol, fmaf(adt, fabsf(L.k1[0]), fabsf(L.tau_seg.hi)), atol);
    if (!(e == e) || isinf(e)) {
      L.status |= JSH_ST_NAN;
      goto abort;
    }
    if (e > 1.0f) {
      const float f = 0.9f * __powf(e, -1.0f / 3.0f);
      L.dt = h * (f > 0.2f ? f : 0.2f);
      if (max_dt != 0.f && fabsf(L.dt) > max_dt) L.dt = max_dt;
      L.rej++;
      if (++L.fails >= dp::FAIL_LIMIT) {
        L.status |= JSH_ST_FAIL_LIMIT;
        goto abort;
      }
      return;
    }
    // landing on the optically thick depth (as the panels)
    if (L.first_seg < 0 && L.tau_seg.hi < L.thick_left && L.tau_seg.hi + inc > 1.25f * L.thick_left) {
      L.dt = h * fmaxf((1.1f * L.thick_left - L.tau_seg.hi) / inc, 0.01f);
      L.last = false;
      L.rej++;
      if (++L.fails >= dp::FAIL_LIMIT) {
        L.status |= JSH_ST_FAIL_LIMIT;
        goto abort;
      }
      return;
    }
    const DF t_prev = L.t;
    const DF t_new = L.last ? L.length : df_add(L.t, h);
    if (t_new.hi == t_prev.hi && t_new.lo == t_prev.lo) {
      L.status |= JSH_ST_DT_UNDERFLOW;
      goto abort;
    }
    L.t = t_new;
    L.bx = df_axpy_round(t_new, DF{R.mix.dhi[0], R.mix.dlo[0]}, L.p0x);
    L.by = df_axpy_round(t_new, DF{R.mix.dhi[1], R.mix.dlo[1]}, L.p0y);
    L.bz = df_axpy_round(t_new, DF{R.mix.dhi[2], R.mix.dlo[2]}, L.p0z);
    L.fails = 0;
    L.acc++;
    if (e < 0.5f) {
      const float ee = e > 0.00032f ? e : 0.00032f;
      L.dt = h * (0.9f * __powf(ee, -0.2f));
      if (max_dt != 0.f && fabsf(L.dt) > max_dt) L.dt = max_dt;
    }
    const DF tau_prev = L.tau_seg;
    L.tau_seg = df_add(L.tau_seg, inc);
    if (L.first_seg < 0 && L.tau_seg.hi >= L.thick_left) {
      L.first_seg = L.seg;
      L.t_first = df_val(t_new);
    }
    if (L.tau_seg.hi > R.mix.tau_max_hi || (L.tau_seg.hi == R.mix.tau_max_hi && L.tau_seg.lo >= R.mix.tau_max_lo)) {
      L.status |= JSH_ST_TAU_CROSSED;
      const double t_old = df_val(t_prev);
      double tc = crossing_time(df_val(tau_prev), t_old, (double)h, h, K(0, 0), K(2, 0), K(3, 0), K(4, 0),
                                K(5, 0), K(6, 0), inc, R.P.tau_max, R.P.tau_precision);
      if (tc < 0.0) {
        // the reference keeps bisecting; stop at the last bracket's midpoint
        L.status |= JSH_ST_BISECT_LIMIT;
        tc = t_old + 0.5 * (double)h;
      }
      if (L.first_seg < 0 || (L.first_seg == L.seg && tc < L.t_first)) {
        L.first_seg = L.seg;
        L.t_first = tc;
      }
      L.nseg = L.seg + 1;
      L.tau_bg += df_val(L.tau_seg);
      L.thick += L.length_cm;
      tau_pass_done<PASS>(L, reqs, part, T);
      return;
    }
    L.k1[0] = K(6, 0);
    return;
  }

segment_done : {
  L.tau_bg += df_val(L.tau_seg);
  L.thick += L.length_cm;
  if (L.seg + 1 < L.nseg) {
    L.seg++;
    begin_tau_segment(L, R, R.hits[L.h]);
    return;
  }
  tau_pass_done<PASS>(L, reqs, part, T);
  return;
}

abort:
  L.tau_bg += df_val(L.tau_seg);
  L.thick += L.length_cm;
  lane_finish(L, reqs, T);
}

// One step of an active lane's tau pass: a quadrature panel for the smooth
// benchmark family (helical conical B and BK n in the plasma frame, flat
// flow), a Dormand-Prince attempt otherwise.  The choice belongs to the
// request, so every build of the kernels gives the same bits.
template <int PASS, bool GENERAL, int W>
__device__ __forceinline__ void tau_step(Lane& L, const JshRequest* __restrict__ reqs, const Stages<1, W>& K1,
                                         int part, Tally& T) {
  if (!GENERAL || reqs[L.r].mix.helical_log) tau_panel_step<PASS, GENERAL>(L, reqs, part, T);
  else tau_dopri_step<PASS, GENERAL, W>(L, reqs, K1, part, T);
}

// ------------------------------------------------------- I / IQUV pass
// One Dormand-Prince attempt (or a segment transition) of an active lane in
// its I/IQUV pass, towards the observer.  The arithmetic is the same in
// every form (static, single-kernel, split), so the images are bitwise the
// same.
template <bool FULL, int PASS, bool GENERAL = true>
__device__ __forceinline__ void lane_step(Lane& L, const JshRequest* __restrict__ reqs,
                                          const Stages<StageWidth<FULL>::NK>& K, Tally& T) {
  constexpr int NK = StageWidth<FULL>::NK;
  constexpr int NX = StageWidth<FULL>::NX;
  const JshRequest& R = reqs[L.r];
  const JshFreqConst F = R.mix.fc[L.f];
  const F3 dirf = f3(R.mix.nl[0], R.mix.nl[1], R.mix.nl[2]);
  // error-norm tolerances in FP32 (the norm needs a few digits; t and dt stay FP64)
  const float atol = F.atol;
  const float rtol = R.mix.rtol;

  if (kFtm && FULL && L.ft) {
    // Faraday-thick mode: its steps follow I and V only, so nothing else
    // keeps them from straddling the narrow features of the field where a
    // ray passes the jet axis (the dip of B_perp, the reversal of the
    // azimuthal field within the approach distance): a step spans at most
    // kFtAxis of the point's distance from the axis.  Where that is under a
    // radian of rotation the full integration is as fast: leave the mode.
    const float cap = kFtAxis * sqrtf(fmaf(L.bx, L.bx, L.by * L.by));
    if (cap * fabsf(L.k1[NK - 1]) < 1.f) {
      L.ft = 0;
      L.ft_cool = kFtCooldown;
      L.init = false;
      L.dt = fminf(L.dt, 1.f / fabsf(L.k1[NK - 1]));
    } else {
      L.dt = fminf(L.dt, cap);
    }
  }
  // integrate_adaptive / adaptive range: finish at exactly t = length (a
  // step that would pass the end is shortened to end there)
  {
    const DF rem = df_sub(L.length, L.t);
    const float remf = rem.hi + rem.lo;
    if (!(remf > 0.f)) goto segment_done;
    L.last = !(L.dt < remf);
    if (L.last) L.dt = remf;
  }
  if (L.nsteps++ >= R.P.max_steps) {
    L.status |= JSH_ST_STEP_LIMIT;
    goto abort;
  }
  {
    const F3 pn = f3(L.bx, L.by, L.bz);
    // frame rotation at the step start: FP32 sincos of the (reduced) angle
    float c0 = 1.f, s0 = 0.f;
    if (FULL) sincosf(L.chi.hi, &s0, &c0);
    const float h = L.dt;
    const bool ft = kFtm && FULL && L.ft;
    float dk[5], cpl = 0.f;  // cpl: Faraday-thick mode, max(|k_Q|, |k_C|) / |lambda| of the last evaluation
    if (!L.init) {
      L.s1 = rhs32<GENERAL>(R, F, FULL, pn, L.x, c0, s0, dk, L.kI1, L.h, (uint32_t)L.f, L.evals0 + L.evals, &L.tri,
                            ft, &cpl);
#pragma unroll
      for (int c = 0; c < NK; ++c) L.k1[c] = dk[c];
      L.evals++;
      L.init = true;
      if (ft) {
        // entry: the transient carried in, d = (q, u) - e^{-i chi} S / lambda,
        // must be small enough that the rotating coupling the mode leaves
        // out of I and V stays within the tolerance
        const float dq = L.x[1] - dk[1], du = L.x[2] - dk[2];
        if (!(cpl * sqrtf(fmaf(dq, dq, du * du)) <= ft_tolerance(L.x[0], rtol, atol))) {
          L.ft = 0;
          L.ft_cool = kFtCooldown;
          L.init = false;
          return;
        }
      }
    }
#pragma unroll
    for (int c = 0; c < NK; ++c) K(0, c) = L.k1[c];
    float inc[NK];
    float smax = L.s1, s7 = 0.f, kI7 = 0.f;
#pragma unroll 1
    for (int s = 1; s < 7; ++s) {
      float acc[NK];
      combine<NK>(s, K, acc);
      float y[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) y[c] = (c < NX) ? fmaf(h, acc[c < NK ? c : 0], L.x[c]) : 0.f;
      float cs = c0, sn = s0;
      if (FULL) {
        float sd, cd;
        __sincosf(h * acc[NK - 1], &sd, &cd);
        cs = c0 * cd - s0 * sd;
        sn = s0 * cd + c0 * sd;
      }
      const float sc = rhs32<GENERAL>(R, F, FULL, pn + dirf * (c_C[s] * h), y, cs, sn, dk, kI7, L.h, (uint32_t)L.f,
                                      L.evals0 + L.evals + (uint32_t)(s - 1), &L.tri, ft, &cpl);
      smax = fmaxf(smax, sc);
      s7 = sc;
      if (ft && s < 6) {
        // Faraday-thick mode: the inner stages' (q, u) slots are free (no
        // stage point uses (q, u)); they keep the stage's k_I and its coupling
        // factor, or +inf where rotation does not outrun absorption a
        // hundredfold (a reversal of the line-of-sight field inside the step,
        // as on rays past the axis of a helical field, breaks the
        // quasi-static picture between the step's ends)
        dk[2] = fabsf(dk[NK - 1]) >= kFtRatio * kI7 ? cpl : INFINITY;
        dk[1] = kI7;
      }
#pragma unroll
      for (int c = 0; c < NK; ++c) K(s, c) = dk[c];
      if (s == 6) {
#pragma unroll
        for (int c = 0; c < NK; ++c) inc[c] = h * acc[c];
      }
    }
    L.evals += 6;
    // embedded error estimate and odeint's default error checker:
    // max_i |err_i| / (atol + rtol (|x_i| + |dt| |x'_i|))
    float err[NK];
#pragma unroll
    for (int c = 0; c < NK; ++c) {
      float a = 0.f;
#pragma unroll
      for (int j = 0; j < 7; ++j) a = fmaf(c_E[j], K(j, c), a);
      err[c] = h * a;
    }
    // FP32 resolution floor: an error estimate below the rounding noise of
    // the terms it is computed from carries no information, so the
    // tolerance never drops below kNoise * h * (their magnitude)
    const float adt = fabsf(h);
    const float floor_ = kNoise * adt * smax;
    float e = 0.f;
    {
      // q', u', V in an optically thick step (optical depth h k_I > 0.01):
      // their source terms are small differences of terms of size ~scale
      // (e_Q - k_Q I, ...) and the rounding noise of their error estimate
      // reaches ~0.7 of the floor, which pins the estimate in odeint's
      // no-growth band [0.5, 1] (95 % of the core rays' steps were there).
      // A 100x floor there (an allowed error of 6e-6 h scale per step, damped
      // by the optical depth in front) took the 512x1024 conical jet's
      // longest item from 4 585 to 2 689 evaluations (10x: 34 % fewer than
      // 1x); against the converged oracle V rose from 3.4e-7 to 1.7e-6 of
      // max I, I and Q stayed.  Optically thin steps keep the 1x floor
      // (their Q/U control is what keeps far rays from stepping over the
      // narrow dip of B_perp where they pass the jet axis).
      const float fl_pol = (adt * fabsf(L.kI1) > 0.01f) ? 100.f * floor_ : floor_;
#pragma unroll
      for (int c = 0; c < NX; ++c) {
        if (ft && (c == 1 || c == 2)) continue;  // (Q, U) is not integrated in the Faraday-thick mode
        const float fl = (c == 0) ? floor_ : fl_pol;
        float r = fabsf(err[c]) / (fmaf(rtol, fmaf(adt, fabsf(L.k1[c]), fabsf(L.x[c])), atol) + fl);
        e = fmaxf(e, r);
      }
      if (ft) {
        // adiabatic condition of the quasi-static part: its lag behind
        // S / lambda, (d/dt (S / lambda)) / lambda, estimated over the step
        // from the lab-frame values at its ends, and the transient's left-out
        // coupling stay within the tolerance; else the step is redone in the
        // full mode (from the same state: (q, u) is the full polarisation in
        // both modes)
        float cs6, sn6;  // the frame at the step's end, as its last stage had it
        {
          float sd, cd;
          __sincosf(inc[NK - 1], &sd, &cd);
          cs6 = c0 * cd - s0 * sd;
          sn6 = s0 * cd + c0 * sd;
        }
        float cpl_max = cpl;
        bool ft_ok = fabsf(K(6, NK - 1)) >= kFtRatio * kI7;
#pragma unroll
        for (int j = 1; j < 6; ++j) cpl_max = fmaxf(cpl_max, K(j, 2));
        ft_ok = ft_ok && cpl_max < INFINITY;
        const float ft_tol = ft_tolerance(L.x[0], rtol, atol);
        const float p0r = c0 * K(0, 1) - s0 * K(0, 2), p0i = s0 * K(0, 1) + c0 * K(0, 2);
        const float p6r = cs6 * K(6, 1) - sn6 * K(6, 2), p6i = sn6 * K(6, 1) + cs6 * K(6, 2);
        const float dr = p6r - p0r, di = p6i - p0i;
        const float lam = sqrtf(fmaf(kI7, kI7, K(6, NK - 1) * K(6, NK - 1)));
        const float dq = L.x[1] - K(0, 1), du = L.x[2] - K(0, 2);
        if (!ft_ok || !(sqrtf(fmaf(dr, dr, di * di)) <= adt * lam * ft_tol) ||
            !(cpl_max * sqrtf(fmaf(dq, dq, du * du)) <= ft_tol)) {
          L.ft = 0;
          L.ft_cool = kFtCooldown;
          L.init = false;
          L.dt = fminf(h, 1.f / fabsf(L.k1[NK - 1]));
          return;
        }
      }
      if (FULL && !ft) {
        // a rotation error d chi moves (Q, U) by P d chi; the lab-frame norm
        // of the reference would compare that with rtol (P + h |dQ/dt|),
        // and |dQ/dt| ~ k_F P there
        float P = sqrtf(fmaf(L.x[1], L.x[1], L.x[2] * L.x[2]));
        e = fmaxf(e, fabsf(err[NK - 1]) * P / (fmaf(rtol * P, fmaf(adt, fabsf(L.k1[NK - 1]), 1.f), atol) + floor_));
      }
    }
    if (!(e == e) || isinf(e)) {
      L.status |= JSH_ST_NAN;
      goto abort;
    }
    if (e > 1.0f) {
      float f = 0.9f * __powf(e, -1.0f / 3.0f);
      L.dt = h * (f > 0.2f ? f : 0.2f);
      L.rej++;
      if (++L.fails >= dp::FAIL_LIMIT) {
        L.status |= JSH_ST_FAIL_LIMIT;
        goto abort;
      }
      return;
    }
    // accept
    const DF t_prev = L.t;
    const DF t_new = L.last ? L.length : df_add(L.t, h);
    if (t_new.hi == t_prev.hi && t_new.lo == t_prev.lo) {
      L.status |= JSH_ST_DT_UNDERFLOW;
      goto abort;
    }
    L.t = t_new;
    L.bx = df_axpy_round(t_new, DF{-R.mix.dhi[0], -R.mix.dlo[0]}, L.p0x);
    L.by = df_axpy_round(t_new, DF{-R.mix.dhi[1], -R.mix.dlo[1]}, L.p0y);
    L.bz = df_axpy_round(t_new, DF{-R.mix.dhi[2], -R.mix.dlo[2]}, L.p0z);
    L.fails = 0;
    L.acc++;
    if (e < 0.5f) {
      float ee = e > 0.00032f ? e : 0.00032f;
      L.dt = h * (0.9f * __powf(ee, -0.2f));
    }
    float qn = 0.f, un = 0.f;
    if (ft) {
      // quasi-static part at the end plus the transient, decayed by the
      // step's optical depth (h sum b_j k_I,j over the stages)
      float btau = c_B[0] * L.kI1;
#pragma unroll
      for (int j = 1; j < 6; ++j) btau = fmaf(c_B[j], K(j, 1), btau);
      const float decay = expf(-h * btau);
      qn = fmaf(L.x[1] - K(0, 1), decay, K(6, 1));
      un = fmaf(L.x[2] - K(0, 2), decay, K(6, 2));
    }
#pragma unroll
    for (int c = 0; c < NX; ++c) L.x[c] += inc[c];
    if (ft) {
      L.x[1] = qn;
      L.x[2] = un;
    }
    if (FULL) {
      L.chi = df_add(L.chi, inc[NK - 1]);
      if (fabsf(L.chi.hi) > 3.14159265f) {
        // subtract k 2 pi exactly: 2 pi = c_hi + c_lo, k c_hi = p + pe
        const float k = rintf(L.chi.hi * 0.159154943f);
        const float c_hi = 6.28318548f, c_lo = -1.74845553e-7f;
        const float pr = k * c_hi, pe = fmaf(k, c_hi, -pr);
        L.chi = df_add(df_add(L.chi, -pr), -fmaf(k, c_lo, pe));
      }
    }
#pragma unroll
    for (int c = 0; c < NK; ++c) L.k1[c] = K(6, c);
    L.s1 = s7;
    L.kI1 = kI7;
    if (kFtm && FULL && !ft) {
      // rotation outruns absorption a hundredfold and turns (q, u) by a
      // noticeable angle per step: try the Faraday-thick mode, whose steps
      // follow I and V, if the transient it would carry looks small enough.
      // The estimate needs no evaluation: this step's last one gives the
      // rotating-frame source e^{-i chi} S = (q, u)' + k_I (q, u), so the
      // quasi-static value and the transient d = (q, u) - e^{-i chi} S / lambda
      // follow, and |d| k_I / |lambda| stands in for the left-out coupling
      // (k_Q, k_C < k_I for synchrotron gas; the first evaluation in the mode
      // checks the entry with the coefficients themselves).
      const float kF = L.k1[NK - 1];
      if (L.ft_cool) L.ft_cool--;
      else if (fabsf(kF) >= kFtRatio * kI7 && fabsf(kF) * h >= 0.01f) {
        const float sr = fmaf(kI7, L.x[1], L.k1[1]), si = fmaf(kI7, L.x[2], L.k1[2]);
        const float il = __fdividef(1.f, fmaf(kI7, kI7, kF * kF));  // an estimate: the fast reciprocal will do
        const float dq = L.x[1] - fmaf(sr, kI7, -si * kF) * il, du = L.x[2] - fmaf(sr, kF, si * kI7) * il;
        const float tol = ft_tolerance(L.x[0], rtol, atol);
        if (kI7 * kI7 * il * fmaf(dq, dq, du * du) <= tol * tol) {
          L.ft = 1;
          L.init = false;
          L.ft_back = 0;
        } else {
          // back off: 16, 32, 64, 128, then 255 steps between estimates
          L.ft_cool = (uint8_t)min(255, kFtRetry << L.ft_back);
          if (L.ft_back < 4) L.ft_back++;
        }
      }
    }
    return;
  }

segment_done : {
  if (L.seg > 0) {
    L.seg--;
    begin_iquv_segment(L, R, R.hits[L.h]);
    return;
  }
  if (PASS == PASS_IQUV) {
    lane_finish_iquv(L, reqs, T);
    return;
  }
  lane_finish(L, reqs, T);
  return;
}

abort:
  if (PASS == PASS_IQUV) {
    lane_finish_iquv(L, reqs, T);
    return;
  }
  lane_finish(L, reqs, T);
}

// One step of an active lane in whichever pass it is.
template <bool FULL, int PASS, bool GENERAL = true>
__device__ __forceinline__ void lane_advance(Lane& L, const JshRequest* __restrict__ reqs,
                                             const Stages<StageWidth<FULL>::NK>& K, Tally& T, int part = 0) {
  if (PASS == PASS_BOTH && L.phase == PH_TAU)
    tau_step<PASS, GENERAL, 7 * StageWidth<FULL>::NK>(L, reqs, Stages<1, 7 * StageWidth<FULL>::NK>{K.t}, part, T);
  else lane_step<FULL, PASS, GENERAL>(L, reqs, K, T);
}

// ------------------------------------------------------------- ranking
// Heaviest-first order of the hit rays for the persistent schedule.  A ray's
// cost grows with its optical depth (up to the optically thick start of the
// IQUV pass): rays through the core take thousands of steps, rays far out a
// few hundred.  So each ray's optical depth at the request's first
// frequency is estimated (4-point Gauss-Legendre over each segment, the FP32
// coefficients), bucketed by factors of 2 and counting-sorted in descending
// order; the queue then hands out the heaviest rays first and they run while
// the bulk fills the GPU, instead of starting late and setting the render's
// makespan.
__global__ void __launch_bounds__(256) rank_cost_kernel(const JshRequest* __restrict__ reqs) {
  __shared__ uint32_t hist[JSH_RANK_BUCKETS];
  const JshRequest& R = reqs[blockIdx.y];
  for (int b = threadIdx.x; b < JSH_RANK_BUCKETS; b += blockDim.x) hist[b] = 0;
  __syncthreads();
  const uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h < *R.n_hit) {
    const JshHit& H = R.hits[h];
    const JshFreqConst F = R.mix.fc[0];
    const float xk[4] = {0.0694318442f, 0.330009478f, 0.669990522f, 0.930568156f};
    const float wk[4] = {0.173927423f, 0.326072577f, 0.326072577f, 0.173927423f};
    float tau = 0.f;
    for (int s = 0; s < H.nseg && s < 2; ++s) {
      const F3 a = f3((float)(H.seg[s][0] * INV_PC), (float)(H.seg[s][1] * INV_PC), (float)(H.seg[s][2] * INV_PC));
      const F3 b = f3((float)(H.seg[s][3] * INV_PC), (float)(H.seg[s][4] * INV_PC), (float)(H.seg[s][5] * INV_PC));
      const F3 d = b - a;
      float acc = 0.f;
#pragma unroll 1
      for (int k = 0; k < 4; ++k) {
        Coef32 c;
        coef32_rt(R, F, a + d * xk[k], COEF_KI, c);
        acc = fmaf(wk[k], c.kI, acc);
      }
      tau = fmaf(acc, sqrtf(fdot(d, d)), tau);
    }
    int key = 0;
    if (tau > 0.f && tau < INFINITY) key = min(max((int)floorf(__log2f(tau)) + 40, 1), JSH_RANK_BUCKETS - 1);
    R.key[h] = (uint8_t)key;
    atomicAdd(&hist[key], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < JSH_RANK_BUCKETS; b += blockDim.x)
    if (hist[b]) atomicAdd(&R.buckets[b], hist[b]);
}

// Start of each bucket in descending bucket order (one thread per request),
// and the size of the deep prefix: the rays of buckets >= deep_key (every
// ray for deep_key <= 0).
__global__ void rank_prefix_kernel(const JshRequest* __restrict__ reqs, int deep_key) {
  const JshRequest& R = reqs[blockIdx.x];
  if (threadIdx.x != 0) return;
  uint32_t run = 0, deep = 0;
  for (int b = JSH_RANK_BUCKETS - 1; b >= 0; --b) {
    R.buckets[JSH_RANK_BUCKETS + b] = run;
    run += R.buckets[b];
    if (b == deep_key) deep = run;
  }
  R.buckets[JSH_RANK_DEEP] = deep_key > 0 ? deep : run;
}

// order[position] = hit index; the lanes of a warp with the same bucket take
// consecutive positions with one atomic.
__global__ void __launch_bounds__(256) rank_scatter_kernel(const JshRequest* __restrict__ reqs) {
  const JshRequest& R = reqs[blockIdx.y];
  const uint32_t h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= *R.n_hit) return;
  const int key = R.key[h];
  const unsigned peers = __match_any_sync(__activemask(), key);
  const int leader = __ffs(peers) - 1;
  const unsigned lane = threadIdx.x & 31u;
  uint32_t base = 0;
  if ((int)lane == leader) base = atomicAdd(&R.buckets[JSH_RANK_BUCKETS + key], (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  R.order[base + __popc(peers & ((1u << lane) - 1u))] = h;
}

// One thread per work item, stepped to completion.
template <bool FULL>
__global__ void __launch_bounds__(128) transfer_static_mixed_kernel(const JshRequest* __restrict__ reqs,
                                                                     int n_req) {
  __shared__ unsigned long long base[JSH_MAX_BATCH + 1];
  extern __shared__ float ksh[];
  batch_prefix(reqs, n_req, base);
  const unsigned long long w = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  const Stages<FULL ? 5 : 1> K{ksh + threadIdx.x * (FULL ? 35 : 7)};
  Tally T = tally_new();
  if (w < base[n_req]) {
    Lane L;
    lane_start(L, reqs, base, n_req, w, false);
    while (L.phase != PH_IDLE) lane_advance<FULL, PASS_BOTH>(L, reqs, K, T);
  }
  tally_flush(T, reqs);
}

// Persistent CTAs: each warp keeps 32 lanes busy, refilling idle lanes from
// the global queue when at least `refill` of them are idle.  COMPACT builds
// the kernel for at most 128 threads and 3 resident CTAs per SM, which caps
// it at 168 registers (154 used, no spills) instead of 198: 12 instead of 10
// resident warps per SM, more latency hiding for the bulk of short rays at
// the price of issue slots for the long ones; the autotuner picks.
template <bool FULL, bool COMPACT>
__global__ void __launch_bounds__(COMPACT ? 128 : 256, COMPACT ? 3 : 1)
    transfer_persistent_mixed_kernel(const JshRequest* __restrict__ reqs, int n_req, unsigned long long* queue,
                                     int refill) {
  __shared__ unsigned long long base[JSH_MAX_BATCH + 1];
  extern __shared__ float ksh[];
  batch_prefix(reqs, n_req, base);
  const Stages<FULL ? 5 : 1> K{ksh + threadIdx.x * (FULL ? 35 : 7)};
  const unsigned long long total = base[n_req];
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  Lane L;
  L.phase = PH_IDLE;
  Tally T = tally_new();
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
        if (w < total) lane_start(L, reqs, base, n_req, w, true);
      }
    }
    unsigned active = __ballot_sync(0xffffffffu, L.phase != PH_IDLE);
    if (active == 0) {
      if (exhausted) break;
      continue;
    }
    if (L.phase != PH_IDLE) lane_advance<FULL, PASS_BOTH>(L, reqs, K, T);
  }
  tally_flush(T, reqs);
}

// ------------------------------------------------------------ split form
// The persistent schedule's default form runs the passes in two kernels:
// every item's tau pass first (one stage component, k_I only: a short
// right-hand side, few registers, many resident warps, and no warp whose
// lanes mix tau and IQUV code), then the I/IQUV pass of the items that need
// one, ranked by the optical depth it integrates through.

// Work items of part `part` of the ranked rays over the batch (exclusive
// prefix in shared memory): part 0 the deep prefix (every ray when the
// passes are not overlapped), part 1 the rays after it.
__device__ __forceinline__ void tau_prefix(const JshRequest* __restrict__ reqs, int n_req, int part,
                                           unsigned long long* base) {
  if (threadIdx.x == 0) {
    unsigned long long acc = 0;
    for (int r = 0; r < n_req; ++r) {
      base[r] = acc;
      const uint32_t deep = reqs[r].buckets[JSH_RANK_DEEP];
      const uint32_t rays = part ? *reqs[r].n_hit - deep : deep;
      acc += (unsigned long long)rays * (unsigned long long)reqs[r].n_nu;
    }
    base[n_req] = acc;
  }
  __syncthreads();
}

// Tau kernel: persistent CTAs, lanes refilled from the ranked queue (the
// same order as the single-kernel form), each item's tau pass to its end,
// over the rays of part `part`.
// GENERAL = false: the build for batches of the fused benchmark family
// alone (80 registers, 24 resident warps per SM, against 128 and 16).
template <bool GENERAL>
__global__ void __launch_bounds__(256, GENERAL ? 2 : 3) transfer_tau_kernel(const JshRequest* __restrict__ reqs,
                                                                          int n_req, unsigned long long* queue,
                                                                          int refill, int part) {
  __shared__ unsigned long long base[JSH_MAX_BATCH + 1];
  extern __shared__ float ksh[];
  tau_prefix(reqs, n_req, part, base);
  const Stages<1> K1{ksh + threadIdx.x * 7};
  const unsigned long long total = base[n_req];
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  Lane L;
  L.phase = PH_IDLE;
  Tally T = tally_new();
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
        if (w < total) lane_start(L, reqs, base, n_req, w, true, part);
      }
    }
    unsigned active = __ballot_sync(0xffffffffu, L.phase != PH_IDLE);
    if (active == 0) {
      if (exhausted) break;
      continue;
    }
    if (L.phase != PH_IDLE) tau_step<PASS_TAU, GENERAL>(L, reqs, K1, part, T);
  }
  tally_flush(T, reqs);
}

// Cost histogram of part `part`'s emitted items of request blockIdx.y
// (grid-stride).
__global__ void __launch_bounds__(256) iquv_hist_kernel(const JshRequest* __restrict__ reqs, int part) {
  __shared__ uint32_t hist[JSH_RANK_BUCKETS];
  const JshRequest& R = reqs[blockIdx.y];
  for (int b = threadIdx.x; b < JSH_RANK_BUCKETS; b += blockDim.x) hist[b] = 0;
  __syncthreads();
  const uint32_t n = R.iq_count[part], o = iq_first(R, part);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(&hist[R.iq_items[o + i].key], 1u);
  __syncthreads();
  uint32_t* bk = R.iq_buckets + 2 * JSH_RANK_BUCKETS * part;
  for (int b = threadIdx.x; b < JSH_RANK_BUCKETS; b += blockDim.x)
    if (hist[b]) atomicAdd(&bk[b], hist[b]);
}

// Start of each cost bucket in descending order (one thread per request).
__global__ void iquv_prefix_kernel(const JshRequest* __restrict__ reqs, int part) {
  const JshRequest& R = reqs[blockIdx.x];
  if (threadIdx.x != 0) return;
  uint32_t* bk = R.iq_buckets + 2 * JSH_RANK_BUCKETS * part;
  uint32_t run = 0;
  for (int b = JSH_RANK_BUCKETS - 1; b >= 0; --b) {
    bk[JSH_RANK_BUCKETS + b] = run;
    run += bk[b];
  }
}

// iq_order[first + position] = emitted item (absolute slot); lanes with the
// same bucket take consecutive positions with one atomic.
__global__ void __launch_bounds__(256) iquv_scatter_kernel(const JshRequest* __restrict__ reqs, int part) {
  const JshRequest& R = reqs[blockIdx.y];
  const uint32_t n = R.iq_count[part], o = iq_first(R, part);
  uint32_t* bk = R.iq_buckets + 2 * JSH_RANK_BUCKETS * part;
  const unsigned lane = threadIdx.x & 31u;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int key = R.iq_items[o + i].key;
    const unsigned peers = __match_any_sync(__activemask(), key);
    const int leader = __ffs(peers) - 1;
    uint32_t b = 0;
    if ((int)lane == leader) b = atomicAdd(&bk[JSH_RANK_BUCKETS + key], (uint32_t)__popc(peers));
    b = __shfl_sync(peers, b, leader);
    R.iq_order[o + b + __popc(peers & ((1u << lane) - 1u))] = o + i;
  }
}

// Exclusive prefix of part `part`'s emitted items over the batch, in shared
// memory.
__device__ __forceinline__ void iquv_prefix(const JshRequest* __restrict__ reqs, int n_req, int part,
                                            unsigned long long* base) {
  if (threadIdx.x == 0) {
    unsigned long long acc = 0;
    for (int r = 0; r < n_req; ++r) {
      base[r] = acc;
      acc += (unsigned long long)reqs[r].iq_count[part];
    }
    base[n_req] = acc;
  }
  __syncthreads();
}

// IQUV kernel: persistent CTAs over the ranked emitted items (COMPACT: the
// register-capped build, as for the single-kernel form).
template <bool FULL, bool COMPACT, bool GENERAL>
__global__ void __launch_bounds__(COMPACT ? 128 : 256, COMPACT ? 3 : 1)
    transfer_iquv_kernel(const JshRequest* __restrict__ reqs, int n_req, unsigned long long* queue, int refill,
                         int part) {
  __shared__ unsigned long long base[JSH_MAX_BATCH + 1];
  extern __shared__ float ksh[];
  iquv_prefix(reqs, n_req, part, base);
  const Stages<FULL ? 5 : 1> K{ksh + threadIdx.x * (FULL ? 35 : 7)};
  const unsigned long long total = base[n_req];
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  Lane L;
  L.phase = PH_IDLE;
  Tally T = tally_new();
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
        if (w < total) lane_start_iquv(L, reqs, base, n_req, w, part);
      }
    }
    unsigned active = __ballot_sync(0xffffffffu, L.phase != PH_IDLE);
    if (active == 0) {
      if (exhausted) break;
      continue;
    }
    if (L.phase != PH_IDLE) lane_step<FULL, PASS_IQUV, GENERAL>(L, reqs, K, T);
  }
  tally_flush(T, reqs);
}

template <bool FULL>
constexpr size_t stage_smem(int block) {
  return sizeof(float) * 7 * (FULL ? 5 : 1) * (size_t)block;
}

// Resident CTAs per SM of the IQUV kernel / the single-kernel form.
int occupancy_mixed(bool split, bool full, int block_size, bool compact) {
  int n = 0;
  if (compact && block_size > 128) return 0;
  const size_t sm = full ? stage_smem<true>(block_size) : stage_smem<false>(block_size);
#define JSH_OCC(kernel) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block_size, sm)
  if (split) {
    // the general build bounds both (it holds at least the fused one's registers)
    if (compact) {
      if (full) JSH_OCC((transfer_iquv_kernel<true, true, true>));
      else JSH_OCC((transfer_iquv_kernel<false, true, true>));
    } else {
      if (full) JSH_OCC((transfer_iquv_kernel<true, false, true>));
      else JSH_OCC((transfer_iquv_kernel<false, false, true>));
    }
  } else {
    if (compact) {
      if (full) JSH_OCC((transfer_persistent_mixed_kernel<true, true>));
      else JSH_OCC((transfer_persistent_mixed_kernel<false, true>));
    } else {
      if (full) JSH_OCC((transfer_persistent_mixed_kernel<true, false>));
      else JSH_OCC((transfer_persistent_mixed_kernel<false, false>));
    }
  }
#undef JSH_OCC
  return n;
}

}  // namespace

}  // namespace jsh

using namespace jsh;

namespace jsh {
namespace {

// Registers a warp of `kernel` holds (allocated in units of 256), looked up
// once per kernel.
template <typename K>
int warp_regs(K kernel) {
  static std::mutex mu;
  static std::unordered_map<const void*, int> known;
  std::lock_guard<std::mutex> lock(mu);
  auto it = known.find((const void*)kernel);
  if (it != known.end()) return it->second;
  cudaFuncAttributes a;
  const int w = cudaFuncGetAttributes(&a, kernel) == cudaSuccess ? (a.numRegs * 32 + 255) / 256 * 256 : 255 * 32;
  known[(const void*)kernel] = w;
  return w;
}

// Launch with a per-launch scheduling priority (the overlapped deep chain).
template <typename... KArgs, typename... Args>
cudaError_t launch_prio(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                        int prio, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = prio;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// IQUV kernel instantiation of a launch.
using IquvKernel = void (*)(const JshRequest*, int, unsigned long long*, int, int);
IquvKernel iquv_kernel(bool full, bool compact, bool fused) {
  if (fused) {
    if (compact) return full ? transfer_iquv_kernel<true, true, false> : transfer_iquv_kernel<false, true, false>;
    return full ? transfer_iquv_kernel<true, false, false> : transfer_iquv_kernel<false, false, false>;
  }
  if (compact) return full ? transfer_iquv_kernel<true, true, true> : transfer_iquv_kernel<false, true, true>;
  return full ? transfer_iquv_kernel<true, false, true> : transfer_iquv_kernel<false, false, true>;
}

// CTAs of the deep chain's IQUV kernel per SM (64 threads each) when the
// passes overlap: room for the deep prefix's longest items from the start,
// the rest of the SM for the other rays' tau kernel.
constexpr int kDeepIquvBlock = 64;
constexpr int kDeepIquvPerSm = 2;

}  // namespace
}  // namespace jsh

#if JSH_FARADAY_THICK_BUILD
#define JSH_LAUNCH_TRANSFER_MIXED jsh_launch_transfer_mixed_ft
#else
#define JSH_LAUNCH_TRANSFER_MIXED jsh_launch_transfer_mixed
#endif
cudaError_t JSH_LAUNCH_TRANSFER_MIXED(const JshRequest* d_reqs, int n_req, int schedule, bool full,
                                      uint64_t max_items, uint64_t max_hits, const JshLaunchShape& shape,
                                      unsigned int* queue, int num_sms, cudaStream_t stream) {
  if (schedule == JSH_SCHED_STATIC) {
    const int bs = 128;
    unsigned blocks = (unsigned)((max_items + bs - 1) / bs);
    if (full)
      transfer_static_mixed_kernel<true><<<blocks, bs, stage_smem<true>(bs), stream>>>(d_reqs, n_req);
    else
      transfer_static_mixed_kernel<false><<<blocks, bs, stage_smem<false>(bs), stream>>>(d_reqs, n_req);
    return cudaGetLastError();
  }
  const bool split = !shape.single;
  const bool overlap = split && shape.overlap_key > 0 && shape.side != nullptr && shape.fork != nullptr;
  if (max_hits > 0) {
    const dim3 g((unsigned)((max_hits + 255) / 256), (unsigned)n_req);
    rank_cost_kernel<<<g, 256, 0, stream>>>(d_reqs);
    rank_prefix_kernel<<<n_req, 32, 0, stream>>>(d_reqs, overlap ? shape.overlap_key : 0);
    rank_scatter_kernel<<<g, 256, 0, stream>>>(d_reqs);
  }
  // queue counters: [0] tau (deep prefix or all) / single-kernel form, [1]
  // its IQUV kernel, [2] and [3] the other rays' tau and IQUV kernels
  unsigned long long* q = (unsigned long long*)queue;
  const uint64_t need = (max_items + 31) / 32 * 32;
  const int rf = shape.refill_threshold;
  int bs = shape.block_size;
  if (bs > (shape.compact ? 128 : 256)) bs = shape.compact ? 128 : 256;
  int per_sm = shape.ctas_per_sm > 0 ? shape.ctas_per_sm : occupancy_mixed(split, full, bs, shape.compact);
  if (per_sm < 1) per_sm = 1;
  unsigned blocks = (unsigned)(num_sms * per_sm);
  if ((uint64_t)blocks * bs > need) blocks = (unsigned)((need + bs - 1) / bs);
  if (blocks == 0) blocks = 1;
  const size_t smem = full ? stage_smem<true>(bs) : stage_smem<false>(bs);
  if (!split) {
    if (shape.marks) cudaEventRecord(shape.marks[2], stream);
    if (shape.compact) {
      if (full) transfer_persistent_mixed_kernel<true, true><<<blocks, bs, smem, stream>>>(d_reqs, n_req, q, rf);
      else transfer_persistent_mixed_kernel<false, true><<<blocks, bs, smem, stream>>>(d_reqs, n_req, q, rf);
    } else {
      if (full) transfer_persistent_mixed_kernel<true, false><<<blocks, bs, smem, stream>>>(d_reqs, n_req, q, rf);
      else transfer_persistent_mixed_kernel<false, false><<<blocks, bs, smem, stream>>>(d_reqs, n_req, q, rf);
    }
    if (shape.marks) cudaEventRecord(shape.marks[3], stream);
    return cudaGetLastError();
  }
  // tau kernel: 256 threads, every CTA it can keep resident (the fused build
  // runs panels only, which keep their sums in registers; the general build
  // keeps Dormand-Prince stages in shared memory)
  const int bt = 256;
  const size_t smem_t = shape.fused ? 0 : stage_smem<false>(bt);
  void (*tau_k)(const JshRequest*, int, unsigned long long*, int, int) =
      shape.fused ? transfer_tau_kernel<false> : transfer_tau_kernel<true>;
  int per_sm_t = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_t, tau_k, bt, smem_t);
  if (per_sm_t < 1) per_sm_t = 1;
  unsigned bl_t = (unsigned)(num_sms * per_sm_t);
  if ((uint64_t)bl_t * bt > need) bl_t = (unsigned)((need + bt - 1) / bt);
  if (bl_t == 0) bl_t = 1;
  const IquvKernel iquv_k = iquv_kernel(full, shape.compact != 0, shape.fused != 0);
  const dim3 gi((unsigned)num_sms, (unsigned)n_req);
  if (!overlap) {
    if (shape.marks) cudaEventRecord(shape.marks[0], stream);
    tau_k<<<bl_t, bt, smem_t, stream>>>(d_reqs, n_req, q, rf, 0);
    if (shape.marks) cudaEventRecord(shape.marks[1], stream);
    iquv_hist_kernel<<<gi, 256, 0, stream>>>(d_reqs, 0);
    iquv_prefix_kernel<<<n_req, 32, 0, stream>>>(d_reqs, 0);
    iquv_scatter_kernel<<<gi, 256, 0, stream>>>(d_reqs, 0);
    if (shape.marks) cudaEventRecord(shape.marks[2], stream);
    iquv_k<<<blocks, bs, smem, stream>>>(d_reqs, n_req, q + 1, rf, 0);
    if (shape.marks) cudaEventRecord(shape.marks[3], stream);
    return cudaGetLastError();
  }
  // Overlapped passes.  Deep chain on `stream`: the deep prefix's tau pass
  // on the whole GPU, its IQUV ranking, then its IQUV kernel at high
  // priority on kDeepIquvPerSm small CTAs per SM.  The other rays' chain on
  // `side` starts when the deep IQUV kernel becomes ready (the fork event
  // follows its ranking), with as many tau CTAs per SM as fit beside the
  // deep IQUV CTAs, so that the deep items start at once and the two chains
  // share every SM.  Neither chain waits on the other inside a kernel.
  static const int prio_hi = [] {
    int least = 0, greatest = 0;
    return cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess ? greatest : 0;
  }();
  const int wr_iquv = warp_regs(iquv_k), wr_tau = warp_regs(tau_k);
  const int deep_warps = kDeepIquvPerSm * kDeepIquvBlock / 32;
  int per_sm_t2 = (65536 - deep_warps * wr_iquv) / ((bt / 32) * wr_tau);
  per_sm_t2 = std::min(std::max(per_sm_t2, 1), per_sm_t);
  if (shape.marks) cudaEventRecord(shape.marks[0], stream);
  cudaError_t e = launch_prio(tau_k, bl_t, bt, smem_t, stream, prio_hi, d_reqs, n_req, q, rf, 0);
  if (e != cudaSuccess) return e;
  iquv_hist_kernel<<<gi, 256, 0, stream>>>(d_reqs, 0);
  iquv_prefix_kernel<<<n_req, 32, 0, stream>>>(d_reqs, 0);
  iquv_scatter_kernel<<<gi, 256, 0, stream>>>(d_reqs, 0);
  e = cudaEventRecord(shape.fork[0], stream);
  if (e != cudaSuccess) return e;
  e = launch_prio(iquv_k, (unsigned)(num_sms * kDeepIquvPerSm), kDeepIquvBlock,
                  full ? stage_smem<true>(kDeepIquvBlock) : stage_smem<false>(kDeepIquvBlock), stream, prio_hi,
                  d_reqs, n_req, q + 1, rf, 0);
  if (e != cudaSuccess) return e;
  e = cudaStreamWaitEvent(shape.side, shape.fork[0], 0);
  if (e != cudaSuccess) return e;
  unsigned bl_t2 = (unsigned)(num_sms * per_sm_t2);
  if ((uint64_t)bl_t2 * bt > need) bl_t2 = (unsigned)((need + bt - 1) / bt);
  if (bl_t2 == 0) bl_t2 = 1;
  tau_k<<<bl_t2, bt, smem_t, shape.side>>>(d_reqs, n_req, q + 2, rf, 1);
  if (shape.marks) cudaEventRecord(shape.marks[1], shape.side);
  iquv_hist_kernel<<<gi, 256, 0, shape.side>>>(d_reqs, 1);
  iquv_prefix_kernel<<<n_req, 32, 0, shape.side>>>(d_reqs, 1);
  iquv_scatter_kernel<<<gi, 256, 0, shape.side>>>(d_reqs, 1);
  if (shape.marks) cudaEventRecord(shape.marks[2], shape.side);
  iquv_k<<<blocks, bs, smem, shape.side>>>(d_reqs, n_req, q + 3, rf, 1);
  e = cudaEventRecord(shape.fork[1], shape.side);
  if (e != cudaSuccess) return e;
  e = cudaStreamWaitEvent(stream, shape.fork[1], 0);
  if (e != cudaSuccess) return e;
  if (shape.marks) cudaEventRecord(shape.marks[3], stream);
  return cudaGetLastError();
}

#if !JSH_FARADAY_THICK_BUILD  // the host functions below are built once
int jsh_queue64_occupancy(int block_size);

int jsh_persistent_occupancy(int precision, bool full, int block_size, bool compact, bool single) {
  if (precision == JSH_PREC_MIXED) return occupancy_mixed(!single, full, block_size, compact);
  return jsh_queue64_occupancy(block_size);
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
  X.dt_max_f = (float)X.dt_max_pc;
  {
    const double d[3] = {req->plane.dx, req->plane.dy, req->plane.dz};
    for (int k = 0; k < 3; ++k) {
      X.dhi[k] = (float)d[k];
      X.dlo[k] = (float)(d[k] - (double)X.dhi[k]);
    }
    X.tau_max_hi = (float)req->P.tau_max;
    X.tau_max_lo = (float)(req->P.tau_max - (double)X.tau_max_hi);
  }
  X.tau_atol = (float)req->P.tau_atol;
  X.tau_rtol = (float)req->P.tau_rtol;
  X.rtol = (float)req->P.rtol;
  X.kq = (float)m.kq_ratio;
  X.eq = (float)m.eq_ratio;
  X.sim_shared = (m.v_kind == JSH_V_SIMULATION && m.n_kind == JSH_N_SIMULATION && m.b_kind == JSH_B_SIMULATION &&
                  m.grid_v == m.grid_b && m.grid_n == m.grid_b)
                     ? 1
                     : 0;
  for (int i = 0; i < 8; ++i) {
    X.vq[i] = (float)m.vp[i];
    X.vq_pc[i] = (float)(m.vp[i] / JSH_PC);
    X.nq[i] = (float)m.np[i];
    X.nq_pc[i] = (float)(m.np[i] / JSH_PC);
    X.bq[i] = (float)m.bp[i];
    X.bq_pc[i] = (float)(m.bp[i] / JSH_PC);
  }
  X.v_dq01 = (float)(m.vp[0] - m.vp[1]);
  X.v_g0m1 = (float)(m.vp[0] - 1.0);
  X.v_cone_oz = (float)m.v_cone_oz;
  X.v_cone_oz_pc = (float)(m.v_cone_oz / JSH_PC);
  X.v_theta = (float)m.v_theta;
  X.v_omc = (float)(2.0 * sin(0.5 * m.vp[2]) * sin(0.5 * m.vp[2]));
  X.sin_pitch = (float)m.sin_pitch;
  X.cos_pitch = (float)m.cos_pitch;
  X.tan_pitch = (float)m.tan_pitch;
  X.b_bessel0 = (float)(m.bp[0] * m.bessel0);
  X.b_bessel1 = (float)(m.bp[0] * m.bessel1);
  // optically thick start of the IQUV pass: the Stokes vector decays at
  // least at rate k_I (1 - |(k_Q, k_U, k_V)| / k_I) along the ray (the
  // symmetric part of the transfer matrix; Faraday terms only rotate), so
  // what enters at optical depth tau_thick is attenuated by exp(-16)
  {
    double p = req->P.full ? std::min(0.95, m.kq_ratio + 0.05) : 0.0;
    double thick = 16.0 / (1.0 - p);
    X.tau_thick = (req->P.flags & JSH_FLAG_IQUV_FROM_TAU_MAX) || !(thick < req->P.tau_max) ? INFINITY : thick;
    // full Stokes: a ray deeper than tau_thick is in local equilibrium well
    // inside it, so its IQUV pass starts at tau_eq = 30 from the equilibrium
    // state x = K^-1 eps of the transfer matrix there (see start_iquv): the
    // part of the ray that start leaves out differs from equilibrium only by
    // the gradients of the source function, attenuated by exp(-(1 - p) 30)
    X.eq_start = (req->P.full && X.tau_thick < INFINITY && kTauEq < X.tau_thick) ? 1 : 0;
    X.tau_eq = X.eq_start ? kTauEq : X.tau_thick;
    X.eq_min = X.eq_start ? std::min(kTauEqMin, X.tau_thick) : X.tau_thick;
  }
  if (m.v_kind == JSH_V_CONST_FLAT) {
    // getG, getD, get_n_los_prime (src/utils.cpp:147-162) in FP64
    double g = m.vp[0];
    double v = JSH_C * sqrt(1. - 1. / (g * g));
    double beta = v / JSH_C;
    double gamma = sqrt(1. / (1. - beta * beta));
    double D = 1. / (gamma * (1. - beta * nz));
    double f = (D + 1.) * (gamma / (gamma + 1.));
    X.v_const = 1;
    X.helical_bk = (m.b_kind == JSH_B_HELICAL_CONICAL && m.n_kind == JSH_N_BK && m.rnd_kind == JSH_RND_NONE) ? 1 : 0;
    const double n0p = m.n_plasma ? m.np[0] : m.np[0] / gamma;
    X.helical_log = (X.helical_bk && m.b_plasma && m.bp[0] != 0.0 && n0p > 0.0) ? 1 : 0;
    if (X.helical_log) {
      X.l2_b0 = (float)log2(fabs(m.bp[0]));
      X.l2_b0D = (float)log2(fabs(m.bp[0]) * D);
      X.l2_n0 = (float)log2(n0p);
      X.pk_h = (float)((s + 1.) / 2.);
      X.b_sign = m.bp[0] > 0.0 ? 1.f : -1.f;
    }
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
    F.atol = (float)(req->P.atol / S);
    F.r_kv = (float)((Av * JSH_PC) / (Ae * JSH_PC / S));
    F.r_ev = (float)((Aev * JSH_PC / S) / (Ak * JSH_PC));
    F.r_kc = (float)((Ac * JSH_PC) * (m.kcr_a * Gnu) / (Ak * JSH_PC));
    if (F.atol == 0.f && req->P.atol > 0.0) F.atol = FLT_MIN;  // below FP32 range: the smallest normal
    const float vals[9] = {F.ak, F.ae, F.av, F.aev, F.af, F.ac, F.r_kv, F.r_ev, F.r_kc};
    for (float x : vals) {
      if (!isfinite(x) || (x != 0.f && fabsf(x) < 1e-30f)) {
        jsh_set_error("frequency %g Hz puts the mixed-precision coefficients outside FP32 range; use FP64", nu);
        return JSH_ERR_INVALID;
      }
    }
  }
  return JSH_OK;
}
#endif  // !JSH_FARADAY_THICK_BUILD
