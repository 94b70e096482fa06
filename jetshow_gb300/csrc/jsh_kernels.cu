// jsh_kernels.cu -- ray generation, hit/compaction and inspection kernels
// and the transfer dispatcher.  The FP64 transfer kernels are in
// jsh_fp64.cu, the mixed-precision ones in jsh_persistent.cu.
#include <cuda_runtime.h>

#include "jsh_fields.cuh"
#include "jsh_launch.h"

using namespace jsh;

namespace {

constexpr int kPlaneThreads = 128;
constexpr int kHitThreads = 256;

// ---------------------------------------------------------------- plane
// pyLogspace by repeated multiplication and the running partial sum are
// sequential recurrences (include/logspace.h:9-33, src/Image.cpp:70-75): one
// thread per request walks them so every value rounds as in the reference.
// Only the two recurrences run here (one FP64 multiply and one add per
// column: an FP64 instruction holds the SM sub-partition's FP64 pipe for
// ~64 cycles on GB300, so the sequential thread is set by their count); the
// running sum goes to along_center and plane_across_kernel turns it into
// the centre, acc - size / 2 (the halving is exact, one rounding as before).
__global__ void plane_along_kernel(const JshRequest* __restrict__ reqs) {
  if (threadIdx.x != 0) return;
  const JshPlane& p = reqs[blockIdx.x].plane;
  double* __restrict__ size = p.along_size;
  double* __restrict__ center = p.along_center;
  const uint64_t n = p.n_along;
  const double base = p.real_base;
  double cur = p.real_start, acc = 0.0;
  for (uint64_t j = 0; j < n; ++j) {
    size[j] = cur;
    acc = (j == 0) ? cur : ad(acc, cur);
    center[j] = acc;
    cur = ml(cur, base);
  }
}

// Column j of the across table: partial sums of n_across/2 copies of the
// column's pixel size, minus half a size (src/Image.cpp:110-126); and the
// column's centre along the plane, its running size sum minus half its size
// (src/Image.cpp:70-75).
__global__ void plane_across_kernel(const JshRequest* __restrict__ reqs) {
  const JshPlane& p = reqs[blockIdx.y].plane;
  uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.n_along) return;
  p.along_center[j] = sb(p.along_center[j], ml(0.5, p.along_size[j]));
  uint64_t nh = p.n_across / 2, na = p.n_along;
  double* __restrict__ pos = p.across_pos;
  double s = ml(p.along_size[j], 1.0);
  double half = ml(0.5, s);
  double a = 0.0;
  for (uint64_t k = 0; k < nh; ++k) {
    a = (k == 0) ? s : ad(a, s);
    pos[k * na + j] = sb(a, half);
  }
}

// ------------------------------------------------------------------ hit
__global__ void hit_kernel(const JshRequest* __restrict__ reqs) {
  const JshRequest& R = reqs[blockIdx.y];
  const JshPlane& p = R.plane;
  uint64_t pix = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = pix < R.npix;
  Hits h;
  h.n = 0;
  h.status = 0;
  if (valid) {
    V3 ro = plane_origin(p, pix / p.n_along, pix % p.n_along);
    geo_hit(R.model, ro, mk(p.dx, p.dy, p.dz), h);
  }
  bool hit = valid && h.n > 0;
  unsigned mask = __ballot_sync(0xffffffffu, hit);
  int lane = threadIdx.x & 31;
  unsigned base = 0;
  if (mask) {
    int leader = __ffs(mask) - 1;
    if (lane == leader) base = atomicAdd(R.n_hit, (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
  }
  if (hit) {
    unsigned slot = base + __popc(mask & ((1u << lane) - 1u));
    JshHit& H = R.hits[slot];
    H.pix = (int64_t)pix;
    H.nseg = h.n;
    H.status = (int32_t)h.status;
#pragma unroll
    for (int s = 0; s < JSH_MAX_SEG; ++s) {
      const Seg& S = h.s[s < h.n ? s : 0];
      H.seg[s][0] = S.in.x;
      H.seg[s][1] = S.in.y;
      H.seg[s][2] = S.in.z;
      H.seg[s][3] = S.out.x;
      H.seg[s][4] = S.out.y;
      H.seg[s][5] = S.out.z;
    }
  } else if (valid) {
    for (int f = 0; f < R.n_nu; ++f) {
      uint64_t q = (uint64_t)f * R.npix + pix;
      if (R.tau) R.tau[q] = 0.0;
      if (R.l) R.l[q] = 0.0;
      if (R.I) R.I[q] = 0.0;
      if (R.Q) R.Q[q] = 0.0;
      if (R.U) R.U[q] = 0.0;
      if (R.V) R.V[q] = 0.0;
      if (R.status) R.status[q] = h.status;
    }
  }
}

__global__ void hit_rays_kernel(JshModel m, const double* __restrict__ orig, const double* __restrict__ dir,
                                int64_t n, int32_t* nseg, double* seg, uint32_t* status) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  V3 ro = mk(orig[3 * i], orig[3 * i + 1], orig[3 * i + 2]);
  V3 rd = vnormalize(mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]));
  Hits h;
  h.n = 0;
  h.status = 0;
  geo_hit(m, ro, rd, h);
  if (nseg) nseg[i] = h.n;
  if (status) status[i] = h.status | (h.n ? JSH_ST_HIT : 0u);
  if (seg) {
    for (int s = 0; s < JSH_MAX_SEG; ++s) {
      double* o = seg + 12 * i + 6 * s;
      if (s < h.n) {
        o[0] = h.s[s].in.x;
        o[1] = h.s[s].in.y;
        o[2] = h.s[s].in.z;
        o[3] = h.s[s].out.x;
        o[4] = h.s[s].out.y;
        o[5] = h.s[s].out.z;
      } else {
        for (int q = 0; q < 6; ++q) o[q] = 0.0;
      }
    }
  }
}

__global__ void plane_rays_kernel(JshPlane p, double* orig, double* sizes) {
  uint64_t pix = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t npix = p.n_across * p.n_along;
  if (pix >= npix) return;
  uint64_t i = pix / p.n_along, j = pix % p.n_along;
  if (orig) {
    V3 o = plane_origin(p, i, j);
    orig[3 * pix] = o.x;
    orig[3 * pix + 1] = o.y;
    orig[3 * pix + 2] = o.z;
  }
  if (sizes) sizes[pix] = p.along_size[j];
}

__global__ void grid_interp_kernel(JshGrid G, int field, const double* zr, int64_t n, double nan_value,
                                   double* out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = grid_value(G, field, zr[2 * i], zr[2 * i + 1], nan_value);
}

// Throughput microbenchmarks: 8 independent dependent chains per thread.
__global__ void peak_fp32_kernel(float* out, int iters, float a) {
  float v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = fmaf(v[i], a, 1e-7f);
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += v[i];
  if (s == 12345.f) out[0] = s;
}

__global__ void peak_mufu_kernel(float* out, int iters) {
  float v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = threadIdx.x * 1e-6f + i * 1e-3f;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float r;
      asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v[i]));
      v[i] = r * 1e-3f;
    }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += v[i];
  if (s == 12345.f) out[0] = s;
}

__global__ void peak_fp64_kernel(double* out, int iters, double a) {
  double v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = fma(v[i], a, 1e-7);
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += v[i];
  if (s == 12345.0) out[0] = s;
}

// ------------------------------------------------------- random cells
__global__ void cells_nearest_kernel(JshCells C, const double* __restrict__ pts, int64_t n, int32_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = cells_nearest64(C, d3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
}

__global__ void random_dir_kernel(uint64_t seed, const uint32_t* __restrict__ keys, int64_t n, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  jsh_random_direction(seed, keys[3 * i], keys[3 * i + 1], keys[3 * i + 2], out + 3 * i);
}

}  // namespace

cudaError_t jsh_run_peaks(int num_sms, double* fp32_tflops, double* mufu_tops, double* fp64_tflops,
                          cudaStream_t stream) {
  void* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, 64);
  if (e != cudaSuccess) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int bs = 256, blocks = num_sms * 8;
  const double threads = (double)bs * blocks;
  const int it32 = 40000, itm = 8000, it64 = 2000;
  float ms = 0.f;
  peak_fp32_kernel<<<blocks, bs, 0, stream>>>((float*)buf, it32 / 2, 0.999999f);  // clocks up
  cudaEventRecord(a, stream);
  peak_fp32_kernel<<<blocks, bs, 0, stream>>>((float*)buf, it32, 0.999999f);
  cudaEventRecord(b, stream);
  cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b);
  if (fp32_tflops) *fp32_tflops = threads * it32 * 8 * 2 / (ms * 1e-3) / 1e12;
  cudaEventRecord(a, stream);
  peak_mufu_kernel<<<blocks, bs, 0, stream>>>((float*)buf, itm);
  cudaEventRecord(b, stream);
  cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b);
  if (mufu_tops) *mufu_tops = threads * itm * 8 / (ms * 1e-3) / 1e12;
  cudaEventRecord(a, stream);
  peak_fp64_kernel<<<blocks, bs, 0, stream>>>((double*)buf, it64, 0.999999);
  cudaEventRecord(b, stream);
  cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b);
  if (fp64_tflops) *fp64_tflops = threads * it64 * 8 * 2 / (ms * 1e-3) / 1e12;
  e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  return e;
}

// Defined in jsh_fp64.cu and jsh_persistent.cu.
cudaError_t jsh_launch_transfer_static64(const JshRequest* d_reqs, int n_req, uint64_t max_items, cudaStream_t stream);
cudaError_t jsh_launch_transfer_persistent64(const JshRequest* d_reqs, int n_req, uint64_t max_items,
                                             const JshLaunchShape& shape, unsigned int* queue, int num_sms,
                                             cudaStream_t stream);
cudaError_t jsh_launch_transfer_mixed(const JshRequest* d_reqs, int n_req, int schedule, bool full,
                                      uint64_t max_items, uint64_t max_hits, const JshLaunchShape& shape,
                                      unsigned int* queue, int num_sms, cudaStream_t stream);
// jsh_persistent_ft.cu: the same launch sequence over the kernels built with
// the Faraday-thick mode
cudaError_t jsh_launch_transfer_mixed_ft(const JshRequest* d_reqs, int n_req, int schedule, bool full,
                                         uint64_t max_items, uint64_t max_hits, const JshLaunchShape& shape,
                                         unsigned int* queue, int num_sms, cudaStream_t stream);

cudaError_t jsh_launch_plane(const JshRequest* d_reqs, int n_req, uint64_t max_along, cudaStream_t stream) {
  if (n_req <= 0) return cudaSuccess;
  plane_along_kernel<<<n_req, 32, 0, stream>>>(d_reqs);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dim3 g((unsigned)((max_along + kPlaneThreads - 1) / kPlaneThreads), (unsigned)n_req);
  plane_across_kernel<<<g, kPlaneThreads, 0, stream>>>(d_reqs);
  return cudaGetLastError();
}

cudaError_t jsh_launch_hit(const JshRequest* d_reqs, int n_req, uint64_t max_pix, cudaStream_t stream) {
  if (n_req <= 0 || max_pix == 0) return cudaSuccess;
  dim3 g((unsigned)((max_pix + kHitThreads - 1) / kHitThreads), (unsigned)n_req);
  hit_kernel<<<g, kHitThreads, 0, stream>>>(d_reqs);
  return cudaGetLastError();
}

cudaError_t jsh_launch_transfer(const JshRequest* d_reqs, int n_req, int precision, int schedule, bool full,
                                uint64_t max_items, uint64_t max_hits, const JshLaunchShape& shape,
                                unsigned int* queue, int num_sms, cudaStream_t stream) {
  if (n_req <= 0 || max_items == 0) return cudaSuccess;
  if (precision == JSH_PREC_MIXED)
    return (full && shape.faraday_thick ? jsh_launch_transfer_mixed_ft : jsh_launch_transfer_mixed)(
        d_reqs, n_req, schedule, full, max_items, max_hits, shape, queue, num_sms, stream);
  if (schedule == JSH_SCHED_PERSISTENT)
    return jsh_launch_transfer_persistent64(d_reqs, n_req, max_items, shape, queue, num_sms, stream);
  return jsh_launch_transfer_static64(d_reqs, n_req, max_items, stream);
}

cudaError_t jsh_launch_hit_rays(const JshModel& model, const double* d_orig, const double* d_dir, int64_t n,
                                int32_t* d_nseg, double* d_seg, uint32_t* d_status, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  hit_rays_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(model, d_orig, d_dir, n, d_nseg, d_seg,
                                                                    d_status);
  return cudaGetLastError();
}

cudaError_t jsh_launch_plane_rays(const JshPlane& plane, double* d_orig, double* d_sizes, cudaStream_t stream) {
  uint64_t npix = plane.n_across * plane.n_along;
  if (npix == 0) return cudaSuccess;
  plane_rays_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, stream>>>(plane, d_orig, d_sizes);
  return cudaGetLastError();
}

cudaError_t jsh_launch_grid_interp(const JshGrid& grid, int field, const double* d_zr, int64_t n, double nan_value,
                                   double* d_out, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  grid_interp_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(grid, field, d_zr, n, nan_value, d_out);
  return cudaGetLastError();
}

cudaError_t jsh_launch_cells_nearest(const JshCells& cells, const double* d_pts, int64_t n, int32_t* d_out,
                                     cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  cells_nearest_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(cells, d_pts, n, d_out);
  return cudaGetLastError();
}

cudaError_t jsh_launch_random_directions(uint64_t seed, const uint32_t* d_keys, int64_t n, double* d_out,
                                         cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  random_dir_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(seed, d_keys, n, d_out);
  return cudaGetLastError();
}
