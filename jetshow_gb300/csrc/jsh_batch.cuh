// jsh_batch.cuh -- mapping of a batch's global work-item index to
// (request, frequency, hit ray), per-request counters and output writes,
// shared by the transfer kernels.
#pragma once

#include "jsh_request.h"
#include "jsh_transfer64.cuh"

namespace jsh {

// Exclusive prefix of work items (n_hit * n_nu) over the batch, in shared memory.
__device__ __forceinline__ void batch_prefix(const JshRequest* __restrict__ reqs, int n_req,
                                             unsigned long long* base) {
  if (threadIdx.x == 0) {
    unsigned long long acc = 0;
    for (int r = 0; r < n_req; ++r) {
      base[r] = acc;
      acc += (unsigned long long)(*reqs[r].n_hit) * (unsigned long long)reqs[r].n_nu;
    }
    base[n_req] = acc;
  }
  __syncthreads();
}

__device__ __forceinline__ int find_request(const unsigned long long* base, int n_req, unsigned long long w) {
  int lo = 0, hi = n_req - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (base[mid] <= w) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Per-request device counters: warp-aggregated when the whole warp works on
// one request, per-lane otherwise.
__device__ __forceinline__ void add_counters(const JshRequest* __restrict__ reqs, int r, bool active,
                                             unsigned long long evals, unsigned long long acc,
                                             unsigned long long rej, unsigned status) {
  int r0 = __shfl_sync(0xffffffffu, r, 0);
  bool same = __all_sync(0xffffffffu, !active || r == r0);
  bool any = __any_sync(0xffffffffu, active);
  if (!any) return;
  if (same) {
    unsigned long long e = warp_sum(active ? evals : 0), a = warp_sum(active ? acc : 0),
                       j = warp_sum(active ? rej : 0);
    unsigned st = __reduce_or_sync(0xffffffffu, active ? status : 0u);
    if ((threadIdx.x & 31) == 0) {
      unsigned long long* c = reqs[r0].counters;
      atomicAdd(&c[0], e);
      atomicAdd(&c[1], a);
      atomicAdd(&c[2], j);
      atomicOr(&c[3], (unsigned long long)st);
    }
  } else if (active) {
    unsigned long long* c = reqs[r].counters;
    atomicAdd(&c[0], evals);
    atomicAdd(&c[1], acc);
    atomicAdd(&c[2], rej);
    atomicOr(&c[3], (unsigned long long)status);
  }
}

__device__ __forceinline__ void write_item(const JshRequest& R, int f, int64_t pix, const ItemOut& o) {
  uint64_t q = (uint64_t)f * R.npix + (uint64_t)pix;
  if (R.tau) R.tau[q] = o.tau;
  if (R.l) R.l[q] = o.l;
  if (R.I) R.I[q] = o.iquv[0];
  if (R.Q) R.Q[q] = o.iquv[1];
  if (R.U) R.U[q] = o.iquv[2];
  if (R.V) R.V[q] = o.iquv[3];
  if (R.status) R.status[q] = o.status;
}

}  // namespace jsh
