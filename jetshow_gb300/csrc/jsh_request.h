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

struct JshParamsDev {
  int32_t n, full, precision, schedule;
  double tau_max, tau_min, dt_max;
  double tau_atol, tau_rtol, atol, rtol, tau_precision;
  int64_t max_steps;
};

struct JshRequest {
  JshModel model;
  JshPlane plane;
  JshParamsDev P;
  JshHit* hits;           // device [npix] (first n_hit valid)
  uint32_t* n_hit;        // device counter written by the hit kernel
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
