// jsh_fp64.cu -- the all-FP64 transfer kernels: one thread per work item
// (static schedule, the plain GPU drop-in) and item-granular dynamic
// scheduling from a global queue.
#include <cuda_runtime.h>

#include "jsh_batch.cuh"
#include "jsh_launch.h"
#include "jsh_transfer64.cuh"

using namespace jsh;

namespace {

// One thread per (request, hit ray, frequency), all FP64.  Items are laid
// out frequency-major within a request so adjacent lanes trace adjacent
// pixels (similar path lengths, less divergence).
__global__ void __launch_bounds__(128) transfer_static64_kernel(const JshRequest* __restrict__ reqs, int n_req) {
  __shared__ unsigned long long base[JSH_MAX_BATCH + 1];
  batch_prefix(reqs, n_req, base);
  unsigned long long w = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool active = w < base[n_req];
  int r = 0;
  Ctl64 tot{0, 0, 0, 0, 0, 0, 0};
  ItemOut o;
  o.status = 0;
  if (active) {
    r = find_request(base, n_req, w);
    const JshRequest& R = reqs[r];
    unsigned long long local = w - base[r];
    unsigned nhit = *R.n_hit;
    int f = (int)(local / nhit);
    unsigned h = (unsigned)(local % nhit);
    const JshHit& H = R.hits[h];
    if (R.P.full) transfer_item64<true>(R.model, R.plane, R.P, H, R.nu[f], f, o, tot);
    else transfer_item64<false>(R.model, R.plane, R.P, H, R.nu[f], f, o, tot);
    if (R.P.flags & JSH_FLAG_COST_MAP) o.l = (double)tot.evals;
    write_item(R, f, H.pix, o);
  }
  add_counters(reqs, r, active, tot.evals, tot.acc, tot.rej, o.status);
}

// FP64 items with dynamic (queue) scheduling at item granularity.
__global__ void __launch_bounds__(128) transfer_queue64_kernel(const JshRequest* __restrict__ reqs, int n_req,
                                                                 unsigned long long* queue) {
  __shared__ unsigned long long base[JSH_MAX_BATCH + 1];
  batch_prefix(reqs, n_req, base);
  const unsigned long long total = base[n_req];
  for (;;) {
    unsigned long long w = atomicAdd(queue, 1ull);
    if (w >= total) break;
    int r = find_request(base, n_req, w);
    const JshRequest& R = reqs[r];
    unsigned long long local = w - base[r];
    unsigned nhit = *R.n_hit;
    int f = (int)(local / nhit);
    const JshHit& H = R.hits[(unsigned)(local % nhit)];
    Ctl64 tot{0, 0, 0, 0, 0, 0, 0};
    ItemOut o;
    if (R.P.full) transfer_item64<true>(R.model, R.plane, R.P, H, R.nu[f], f, o, tot);
    else transfer_item64<false>(R.model, R.plane, R.P, H, R.nu[f], f, o, tot);
    uint64_t q = (uint64_t)f * R.npix + (uint64_t)H.pix;
    if (R.tau) R.tau[q] = o.tau;
    if (R.l) R.l[q] = (R.P.flags & JSH_FLAG_COST_MAP) ? (double)tot.evals : o.l;
    if (R.I) R.I[q] = o.iquv[0];
    if (R.Q) R.Q[q] = o.iquv[1];
    if (R.U) R.U[q] = o.iquv[2];
    if (R.V) R.V[q] = o.iquv[3];
    if (R.status) R.status[q] = o.status;
    atomicAdd(&R.counters[0], (unsigned long long)tot.evals);
    atomicAdd(&R.counters[1], (unsigned long long)tot.acc);
    atomicAdd(&R.counters[2], (unsigned long long)tot.rej);
    atomicOr(&R.counters[3], (unsigned long long)o.status);
  }
}


}  // namespace

cudaError_t jsh_launch_transfer_static64(const JshRequest* d_reqs, int n_req, uint64_t max_items, cudaStream_t stream) {
  const int bs = 128;
  uint64_t blocks = (max_items + bs - 1) / bs;
  transfer_static64_kernel<<<(unsigned)blocks, bs, 0, stream>>>(d_reqs, n_req);
  return cudaGetLastError();
}

cudaError_t jsh_launch_transfer_persistent64(const JshRequest* d_reqs, int n_req, uint64_t max_items,
                                             const JshLaunchShape& shape, unsigned int* queue, int num_sms,
                                             cudaStream_t stream) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transfer_queue64_kernel, 128, 0);
  if (per_sm < 1) per_sm = 1;
  unsigned blocks = (unsigned)(num_sms * per_sm);
  uint64_t need = (max_items + 127) / 128;
  if (blocks > need) blocks = (unsigned)(need ? need : 1);
  transfer_queue64_kernel<<<blocks, 128, 0, stream>>>(d_reqs, n_req, (unsigned long long*)queue);
  return cudaGetLastError();
}

int jsh_queue64_occupancy(int block_size) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, transfer_queue64_kernel, block_size, 0);
  return n;
}


