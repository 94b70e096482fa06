// jsh_cells.cpp -- random cell sets of CellsRandomVectorBField on the host:
// the cells of RandomCellsInSphere::create (src/Cells.cpp:35-47, with the
// point and direction draws of src/utils.cpp:249-312 made counter-based),
// the upload with its nearest-cell bucket grid, and the check entry points.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "jsh_context.h"
#include "jsh_random.h"

namespace {

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

// Squared distance from p to the box [lo, hi] (0 inside) and to its farthest point.
void box_dists(const double* p, const double* lo, const double* hi, double* dmin2, double* dmax2) {
  double a = 0.0, b = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double dl = lo[k] - p[k], dh = p[k] - hi[k];
    const double out = std::max(0.0, std::max(dl, dh));
    const double far = std::max(std::fabs(dl), std::fabs(dh));
    a += out * out;
    b += far * far;
  }
  *dmin2 = a;
  *dmax2 = b;
}

}  // namespace

extern "C" int jsh_cells_generate(int64_t n, double r_min, double r_max, double theta_max, double exponent,
                                  uint64_t seed, double* points, double* directions) {
  if (n < 1 || n > (1LL << 31) - 2 || !points || !directions) {
    jsh_set_error("jsh_cells_generate: n in [1, 2^31 - 2] and both outputs required");
    return JSH_ERR_INVALID;
  }
  if (!std::isfinite(r_min) || !std::isfinite(r_max) || !std::isfinite(theta_max) || !std::isfinite(exponent) ||
      exponent == 3.0) {
    jsh_set_error("jsh_cells_generate: finite arguments and exponent != 3 required");
    return JSH_ERR_INVALID;
  }
  // generate_random_points_sphere (src/utils.cpp:267-312)
  const double c = theta_max > 0 ? cos(theta_max) : 1.0;
  const double pw = 1. / (3.0 - exponent);
  for (int64_t j = 0; j < n; ++j) {
    const JshU4 u = jsh_philox4x32_10(JshU4{(uint32_t)j, JSH_CELL_POINT_KEY, 0u, JSH_STREAM_CELL_POINT}, seed);
    double r = r_min + (r_max - r_min) * jsh_u01(u.x);
    const double phi = 2.0 * JSH_PI * jsh_u01(u.y);
    double uu = (1.0 - c) * (2.0 * jsh_u01(u.z) - 1.0);
    if (uu < 0.0) uu = uu - c;
    else uu = uu + c;
    const double theta = acos(uu);
    r = pow(r, pw);
    points[3 * j] = r * sin(theta) * cos(phi);
    points[3 * j + 1] = r * sin(theta) * sin(phi);
    points[3 * j + 2] = r * cos(theta);
    // generate_random_directions (src/utils.cpp:249-261)
    jsh_random_direction(seed, (uint32_t)j, JSH_CELL_KEY, 0u, directions + 3 * j);
  }
  return JSH_OK;
}

extern "C" int jsh_cells_upload(jsh_ctx* ctx, const double* points, const double* directions, int64_t n,
                                int32_t* cells_id) {
  if (!ctx || !points || !directions || !cells_id || n < 1 || n > (1 << 24)) {
    jsh_set_error("jsh_cells_upload: context, points, directions, id required and 1 <= n <= 2^24");
    return JSH_ERR_INVALID;
  }
  double lo[3], hi[3];
  for (int k = 0; k < 3; ++k) lo[k] = hi[k] = points[k];
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      const double v = points[3 * i + k];
      if (!std::isfinite(v) || !std::isfinite(directions[3 * i + k])) {
        jsh_set_error("cell points and directions must be finite");
        return JSH_ERR_INVALID;
      }
      lo[k] = std::min(lo[k], v);
      hi[k] = std::max(hi[k], v);
    }
  // grid over the box grown by a quarter of its largest side on every side,
  // cubic buckets, about two cells per bucket (at most 64 per axis)
  double ext = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
  if (!(ext > 0)) ext = std::max(1.0, std::fabs(lo[0]) + std::fabs(lo[1]) + std::fabs(lo[2]));
  for (int k = 0; k < 3; ++k) {
    lo[k] -= 0.25 * ext;
    hi[k] += 0.25 * ext;
  }
  const double vol = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
  double h = std::cbrt(vol / std::max(1.0, (double)n / 2.0));
  h = std::max(h, std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]) / 64.0);
  int nb[3];
  for (int k = 0; k < 3; ++k) nb[k] = std::max(1, std::min(64, (int)std::ceil((hi[k] - lo[k]) / h)));
  const int64_t nbk = (int64_t)nb[0] * nb[1] * nb[2];
  std::vector<int32_t> bstart((size_t)nbk + 1, 0), items;
  for (int64_t b = 0; b < nbk; ++b) {
    const int bx = (int)(b % nb[0]), by = (int)((b / nb[0]) % nb[1]), bz = (int)(b / ((int64_t)nb[0] * nb[1]));
    const double blo[3] = {lo[0] + bx * h, lo[1] + by * h, lo[2] + bz * h};
    const double bhi[3] = {blo[0] + h, blo[1] + h, blo[2] + h};
    // every point within the smallest farthest-corner distance can be the
    // nearest somewhere in the bucket; the margin keeps rounding on the safe side
    double dcap = INFINITY;
    for (int64_t i = 0; i < n; ++i) {
      double a, f;
      box_dists(points + 3 * i, blo, bhi, &a, &f);
      dcap = std::min(dcap, f);
    }
    dcap = dcap * (1.0 + 1e-9) + 1e-300;
    for (int64_t i = 0; i < n; ++i) {
      double a, f;
      box_dists(points + 3 * i, blo, bhi, &a, &f);
      if (a <= dcap) items.push_back((int32_t)i);
    }
    bstart[(size_t)b + 1] = (int32_t)items.size();
  }
  std::vector<float> pf((size_t)3 * n), df((size_t)3 * n);
  for (int64_t i = 0; i < 3 * n; ++i) {
    pf[i] = (float)(points[i] / JSH_PC);
    df[i] = (float)directions[i];
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  int id = -1;
  for (int g = 0; g < JSH_MAX_CELL_SETS && id < 0; ++g)
    if (!ctx->cells[g].used) id = g;
  if (id < 0) {
    jsh_set_error("all %d cell-set slots are in use", JSH_MAX_CELL_SETS);
    return JSH_ERR_OOM;
  }
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  const size_t o_p = 0, o_pf = up256(o_p + sizeof(double) * 3 * n), o_d = up256(o_pf + sizeof(float) * 3 * n),
               o_df = up256(o_d + sizeof(double) * 3 * n), o_bs = up256(o_df + sizeof(float) * 3 * n),
               o_it = up256(o_bs + sizeof(int32_t) * (nbk + 1)),
               total = up256(o_it + sizeof(int32_t) * std::max<size_t>(1, items.size()));
  void* mem = nullptr;
  int st = jsh_alloc_device(ctx, total, &mem);
  if (st) return st;
  char* b = (char*)mem;
  cudaError_t e = cudaMemcpy(b + o_p, points, sizeof(double) * 3 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b + o_pf, pf.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b + o_d, directions, sizeof(double) * 3 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b + o_df, df.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b + o_bs, bstart.data(), sizeof(int32_t) * (nbk + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !items.empty())
    e = cudaMemcpy(b + o_it, items.data(), sizeof(int32_t) * items.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    jsh_free_device(ctx, mem, total);
    jsh_set_error("cell-set upload failed: %s", cudaGetErrorString(e));
    return JSH_ERR_CUDA;
  }
  JshCellSlot& S = ctx->cells[id];
  JshCells& V = S.view;
  V.p = (const double*)(b + o_p);
  V.pf = (const float*)(b + o_pf);
  V.dir = (const double*)(b + o_d);
  V.dirf = (const float*)(b + o_df);
  V.bstart = (const int32_t*)(b + o_bs);
  V.bitems = (const int32_t*)(b + o_it);
  V.n = (int32_t)n;
  V.nbx = nb[0];
  V.nby = nb[1];
  V.nbz = nb[2];
  V.x0 = lo[0];
  V.y0 = lo[1];
  V.z0 = lo[2];
  V.h = h;
  V.x0f = (float)(lo[0] / JSH_PC);
  V.y0f = (float)(lo[1] / JSH_PC);
  V.z0f = (float)(lo[2] / JSH_PC);
  V.inv_hf = (float)(JSH_PC / h);
  S.mem = mem;
  S.bytes = total;
  S.used.store(true, std::memory_order_release);
  *cells_id = id;
  return JSH_OK;
}

int jsh_resolve_cells(jsh_ctx* ctx, JshModel* model) {
  if (model->rnd_kind != JSH_RND_CELLS) return JSH_OK;
  if (!ctx) {
    jsh_set_error("random cell sets live in a context; this entry point has none");
    return JSH_ERR_INVALID;
  }
  const int id = model->cells_id;
  if (id < 0 || id >= JSH_MAX_CELL_SETS || !ctx->cells[id].used.load(std::memory_order_acquire)) {
    jsh_set_error("random field refers to cell set %d which is not uploaded", id);
    return JSH_ERR_NOT_FOUND;
  }
  model->cells = ctx->cells[id].view;
  return JSH_OK;
}

extern "C" int jsh_cells_nearest(jsh_ctx* ctx, int32_t cells_id, const double* points, int64_t n, int32_t* out) {
  if (!ctx || (n > 0 && (!points || !out)) || n < 0) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  if (n == 0) return JSH_OK;
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (cells_id < 0 || cells_id >= JSH_MAX_CELL_SETS || !ctx->cells[cells_id].used.load(std::memory_order_acquire)) {
    jsh_set_error("cell set %d is not uploaded", cells_id);
    return JSH_ERR_NOT_FOUND;
  }
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  const size_t o_p = 0, o_o = up256(sizeof(double) * 3 * n), total = up256(o_o + sizeof(int32_t) * n);
  int st = ensure_workspace(ctx, total);
  if (st) return st;
  JSH_CUDA_TRY(cudaEventSynchronize(ctx->ws_ready));
  char* b = (char*)ctx->ws;
  cudaStream_t s = ctx->stream;
  JSH_CUDA_TRY(cudaMemcpyAsync(b + o_p, points, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  JSH_CUDA_TRY(jsh_launch_cells_nearest(ctx->cells[cells_id].view, (const double*)(b + o_p), n, (int32_t*)(b + o_o), s));
  JSH_CUDA_TRY(cudaMemcpyAsync(out, b + o_o, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  JSH_CUDA_TRY(cudaEventRecord(ctx->ws_ready, s));
  JSH_CUDA_TRY(cudaStreamSynchronize(s));
  return JSH_OK;
}

extern "C" int jsh_random_directions(jsh_ctx* ctx, uint64_t seed, const uint32_t* keys, int64_t n, double* out) {
  if (!ctx || (n > 0 && (!keys || !out)) || n < 0) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  if (n == 0) return JSH_OK;
  std::lock_guard<std::mutex> lk(ctx->mu);
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  const size_t o_k = 0, o_o = up256(sizeof(uint32_t) * 3 * n), total = up256(o_o + sizeof(double) * 3 * n);
  int st = ensure_workspace(ctx, total);
  if (st) return st;
  JSH_CUDA_TRY(cudaEventSynchronize(ctx->ws_ready));
  char* b = (char*)ctx->ws;
  cudaStream_t s = ctx->stream;
  JSH_CUDA_TRY(cudaMemcpyAsync(b + o_k, keys, sizeof(uint32_t) * 3 * n, cudaMemcpyHostToDevice, s));
  JSH_CUDA_TRY(jsh_launch_random_directions(seed, (const uint32_t*)(b + o_k), n, (double*)(b + o_o), s));
  JSH_CUDA_TRY(cudaMemcpyAsync(out, b + o_o, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  JSH_CUDA_TRY(cudaEventRecord(ctx->ws_ready, s));
  JSH_CUDA_TRY(cudaStreamSynchronize(s));
  return JSH_OK;
}
