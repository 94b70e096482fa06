// jsh_request.h -- device-visible description of one render request: the
// compiled model and plane, the hit list the hit kernel produces, the
// frequencies, the integration parameters and the output planes.  A batch
// is an array of these; kernels map a global work item to (request, hit
// ray, frequency).
#pragma once

#include "jsh_model.h"

struct JshHit {           // one intersecting pixel (Intersection list)
  int64_t pix;            // flat pixel index i * n_along + j
  int32_t nseg;           // 1 or 2
  int32_t status;         // geometry status bits
  double seg[JSH_MAX_SEG][6];  // {point_in xyz, point_out xyz}
};

// Cost buckets of the heaviest-first ranking (factors of 2 in optical depth).
#define JSH_RANK_BUCKETS 64
// Words of a request's ranking state: bucket counts, bucket cursors, then
// the number of ranked rays in the deep prefix (the rays whose passes run
// ahead of the others when the split form overlaps them; all rays when not).
#define JSH_RANK_DEEP (2 * JSH_RANK_BUCKETS)
#define JSH_RANK_WORDS (2 * JSH_RANK_BUCKETS + 32)
// Words of a request's IQUV ranking state: counts and cursors of the deep
// prefix's emitted items, then those of the other rays' items.
#define JSH_IQ_WORDS (4 * JSH_RANK_BUCKETS)

// Persistent mixed schedule, split form: one work item whose tau pass has
// finished and whose I/IQUV pass is still to run, as the tau kernel hands it
// to the IQUV kernel (32 bytes).  The tau and l planes of the item are
// written already; the IQUV kernel writes I, Q, U, V and the final status.
struct JshIquvItem {
  uint32_t h;          // hit index
  uint16_t f;          // frequency index
  uint8_t key;         // IQUV cost bucket (heaviest-first order)
  uint8_t flags;       // bits 0-1: nseg; bit 2: equilibrium start; bits 3-4: first_seg + 1
  uint32_t status;     // status bits of the tau pass (JSH_ST_IQUV set)
  uint32_t evals;      // right-hand-side evaluations of the tau pass (cost map)
  double tau_bg;       // total optical depth of the tau pass
  double t_first;      // [pc] IQUV start on first_seg (tau_max crossing or optically thick point)
};

struct JshParamsDev {
  int32_t n, full, precision, schedule, flags, pad_;
  double tau_max, tau_min, dt_max;
  double tau_atol, tau_rtol, atol, rtol, tau_precision;
  int64_t max_steps;
};

// Mixed precision, one frequency: folded prefactors of the FP32 coefficient
// algebra (see jsh_fields32.cuh), lengths in pc, intensities in units of
// `scale`.
struct JshFreqConst {
  float ak, ae, av, aev, af, ac, c1, c2;
  double scale;  // S: cgs intensity of one unit of the scaled state
  float atol;    // I/IQUV-pass atol / S
  float r_kv;    // a_V / a_e      (log-domain helical path)
  float r_ev;    // a_eV / a_k
  float r_kc;    // a_C c2 / a_k
};

// Mixed precision, per request.
struct JshMixed {
  int32_t v_const;       // ConstFlat velocity: Doppler factor and aberrated LOS are constants
  int32_t helical_bk;    // ConstFlat V, helical conical B, BK n: the fused field path
  int32_t helical_log;   // ... with B in the plasma frame: the log-domain coefficients
  float l2_b0, l2_b0D;   // log2 |b0|, log2(|b0| D)
  float l2_n0;           // log2 of n0 in the plasma frame (n0 / Gamma if given in the lab)
  float pk_h;            // (s + 1) / 2
  float b_sign;          // sign of b0
  int32_t sim_shared;    // V, N and B all from one grid: one point location per evaluation
  float D, gamma, beta;  // of the constant velocity
  float nlp[3];          // aberrated LOS of the constant velocity
  float nl[3];           // LOS towards the observer (-ray direction)
  float pk;              // (s + 2) / 2
  float kq, eq;          // k_Q / k_I, eta_Q / eta_I
  int32_t eq_start;      // full Stokes: start thick rays at tau_eq in local equilibrium
  double dt_max_pc;      // tau-pass step limit [pc], 0 = none
  double tau_thick;      // optical depth beyond which the truncated part of a ray is negligible
  double tau_eq;         // the tau pass lands a step on this depth; IQUV starts there
                         // (zero state if tau_eq == tau_thick, local equilibrium otherwise)
  double eq_min;         // equilibrium start only for rays at least this deep
  // FP32 copies of the field parameters (q) and of q / pc, and the derived
  // constants the FP32 field laws use: no FP64 operation per evaluation
  float vq[8], vq_pc[8], nq[8], nq_pc[8], bq[8], bq_pc[8];
  float v_dq01, v_g0m1, v_cone_oz, v_cone_oz_pc, v_theta;
  float v_omc;           // SheathCentral: 1 - cos(theta_sheath) = 2 sin^2(theta_sheath / 2)
  float sin_pitch, cos_pitch, tan_pitch, b_bessel0, b_bessel1;
  float tau_atol, tau_rtol, rtol;  // FP32 copies of the step-control tolerances
  float dt_max_f;                  // dt_max_pc in FP32
  float dhi[3], dlo[3];            // ray direction as compensated FP32 pairs
  float tau_max_hi, tau_max_lo;    // tau_max as a compensated FP32 pair
  const JshFreqConst* fc;  // device [n_nu]
};

struct JshRequest {
  JshModel model;
  JshMixed mix;
  JshPlane plane;
  JshParamsDev P;
  JshHit* hits;           // device [npix] (first n_hit valid)
  // persistent mixed schedule: hit rays ranked by estimated cost, heaviest
  // first (order[rank] = hit index), their cost buckets and the ranking
  // state [JSH_RANK_WORDS] (zeroed with the counters)
  uint32_t* order;
  uint8_t* key;
  uint32_t* buckets;
  uint32_t* n_hit;        // device counter written by the hit kernel
  // persistent mixed schedule, split form: items handed from the tau kernel
  // to the IQUV kernel [npix * n_nu], their heaviest-first order, their
  // counts [2] and the IQUV ranking state [JSH_IQ_WORDS] (counts and state
  // zeroed with the counters).  The deep prefix's items fill the array from
  // 0, the other rays' items from n_deep * n_nu (n_deep =
  // buckets[JSH_RANK_DEEP]); iq_order holds absolute item indices.
  JshIquvItem* iq_items;
  uint32_t* iq_order;
  uint32_t* iq_count;
  uint32_t* iq_buckets;
  const double* nu;       // device [n_nu] source-frame frequencies
  int32_t n_nu;
  int32_t reserved;
  uint64_t npix;
  double* tau;            // device output planes [n_nu][npix], any may be NULL
  double* l;
  double* I;
  double* Q;
  double* U;
  double* V;
  uint32_t* status;
  unsigned long long* counters;  // device [4]: rhs evals, accepted, rejected, status OR
};
