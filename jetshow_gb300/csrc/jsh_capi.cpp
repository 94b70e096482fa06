// jsh_capi.cpp -- the blocking and stream-ordered render entry points of the
// C ABI (include/jetshow_capi.h), ray/hit inspection entry points and grid
// upload.  Replaces Observation::run + getImage (src/Observation.cpp:20-46)
// and the ImagePlane/Geometry constructors the bindings call
// (src/pyjetshow.cpp:69-173).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "jsh_quadrature.h"
#include "jsh_context.h"

namespace {

size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

bool all_finite_positive(const double* nu, int n) {
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(nu[i]) || !(nu[i] > 0)) return false;
  return true;
}

}  // namespace

int jsh_alloc_device(jsh_ctx* ctx, size_t bytes, void** p) {
  if (bytes == 0) bytes = 256;
  uint64_t after = ctx->used.fetch_add(bytes) + bytes;
  if (after > ctx->budget) {
    ctx->used.fetch_sub(bytes);
    jsh_set_error("HBM budget exceeded: need %zu more bytes (%llu of %llu in use)", bytes,
                  (unsigned long long)(after - bytes), (unsigned long long)ctx->budget);
    return JSH_ERR_OOM;
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    ctx->used.fetch_sub(bytes);
    cudaGetLastError();
    jsh_set_error("cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? JSH_ERR_OOM : JSH_ERR_CUDA;
  }
  return JSH_OK;
}

void jsh_free_device(jsh_ctx* ctx, void* p, size_t bytes) {
  if (!p) return;
  if (bytes == 0) bytes = 256;
  cudaFree(p);
  ctx->used.fetch_sub(bytes);
}

void jsh_request_layout(uint64_t npix, uint64_t n_along, uint64_t n_across, int32_t n_nu, bool own_outputs,
                        JshRequestLayout* L) {
  size_t o = 0;
  L->off_req = o;
  o = align_up(o + sizeof(JshRequest));
  L->off_counters = o;
  o = align_up(o + 8 * sizeof(unsigned long long));
  L->off_nhit = o;
  o = align_up(o + sizeof(uint32_t));
  L->off_queue = o;
  o = align_up(o + 4 * sizeof(unsigned long long));
  L->off_buckets = o;
  o = align_up(o + sizeof(uint32_t) * JSH_RANK_WORDS);
  L->off_iq_count = o;
  o = align_up(o + 2 * sizeof(uint32_t));
  L->off_iq_buckets = o;
  o = align_up(o + sizeof(uint32_t) * JSH_IQ_WORDS);
  L->off_nu = o;
  o = align_up(o + sizeof(double) * n_nu);
  L->off_fc = o;
  o = align_up(o + sizeof(JshFreqConst) * n_nu);
  L->off_along_size = o;
  o = align_up(o + sizeof(double) * n_along);
  L->off_along_center = o;
  o = align_up(o + sizeof(double) * n_along);
  L->off_across = o;
  o = align_up(o + sizeof(double) * (n_across / 2) * n_along);
  L->off_hits = o;
  o = align_up(o + sizeof(JshHit) * npix);
  L->off_order = o;
  o = align_up(o + sizeof(uint32_t) * npix);
  L->off_key = o;
  o = align_up(o + npix);
  L->off_iq_items = o;
  o = align_up(o + sizeof(JshIquvItem) * npix * (uint64_t)n_nu);
  L->off_iq_order = o;
  o = align_up(o + sizeof(uint32_t) * npix * (uint64_t)n_nu);
  L->own_outputs = own_outputs;
  for (int k = 0; k < 7; ++k) {
    L->off_out[k] = o;
    if (own_outputs) o = align_up(o + (k < 6 ? sizeof(double) : sizeof(uint32_t)) * npix * (uint64_t)n_nu);
  }
  L->total = o;
}

void jsh_bind_request(JshRequest* req, char* base, const JshRequestLayout& L, bool own_outputs) {
  req->counters = (unsigned long long*)(base + L.off_counters);
  req->n_hit = (uint32_t*)(base + L.off_nhit);
  req->nu = (const double*)(base + L.off_nu);
  req->mix.fc = (const JshFreqConst*)(base + L.off_fc);
  req->plane.along_size = (double*)(base + L.off_along_size);
  req->plane.along_center = (double*)(base + L.off_along_center);
  req->plane.across_pos = (double*)(base + L.off_across);
  req->hits = (JshHit*)(base + L.off_hits);
  req->buckets = (uint32_t*)(base + L.off_buckets);
  req->order = (uint32_t*)(base + L.off_order);
  req->key = (uint8_t*)(base + L.off_key);
  req->iq_items = (JshIquvItem*)(base + L.off_iq_items);
  req->iq_order = (uint32_t*)(base + L.off_iq_order);
  req->iq_count = (uint32_t*)(base + L.off_iq_count);
  req->iq_buckets = (uint32_t*)(base + L.off_iq_buckets);
  if (own_outputs) {
    req->tau = (double*)(base + L.off_out[0]);
    req->l = (double*)(base + L.off_out[1]);
    req->I = (double*)(base + L.off_out[2]);
    req->Q = (double*)(base + L.off_out[3]);
    req->U = (double*)(base + L.off_out[4]);
    req->V = (double*)(base + L.off_out[5]);
    req->status = (uint32_t*)(base + L.off_out[6]);
  }
}

int jsh_kernels_per_request(int precision, int schedule, bool single, bool overlap) {
  if (precision == JSH_PREC_MIXED && schedule == JSH_SCHED_PERSISTENT) return single ? 7 : (overlap ? 15 : 11);
  return 4;
}

bool jsh_overlap_passes(const jsh_params* params, const JshLaunchShape& shape, uint64_t items) {
  return params->precision == JSH_PREC_MIXED && params->schedule == JSH_SCHED_PERSISTENT && !shape.single &&
         !(params->flags & JSH_FLAG_SERIAL_PASSES) &&
         ((params->flags & JSH_FLAG_OVERLAP_PASSES) || shape.overlap_key > 0) && items >= JSH_OVERLAP_MIN_ITEMS;
}

JshLaunchShape jsh_effective_shape(const jsh_ctx* ctx, const jsh_params* params) {
  return jsh_params_shape(ctx->shape, params);
}

JshLaunchShape jsh_params_shape(JshLaunchShape s, const jsh_params* params) {
  if (params->block_size > 0) s.block_size = params->block_size;
  if (params->ctas_per_sm > 0) s.ctas_per_sm = params->ctas_per_sm;
  if (params->refill_threshold > 0) s.refill_threshold = params->refill_threshold;
  if (params->flags & JSH_FLAG_COMPACT_REGS) s.compact = 1;
  if (params->flags & JSH_FLAG_SINGLE_KERNEL) s.single = 1;
  s.faraday_thick = (params->flags & JSH_FLAG_FARADAY_THICK) ? 1 : 0;
  if (s.block_size < 32) s.block_size = 32;
  if (s.block_size > 512) s.block_size = 512;
  s.block_size = s.block_size / 32 * 32;
  if (s.refill_threshold < 1) s.refill_threshold = 1;
  if (s.refill_threshold > 32) s.refill_threshold = 32;
  return s;
}

int jsh_prepare_request(jsh_ctx* ctx, const jsh_model_desc* model, const jsh_plane_desc* plane,
                        const jsh_params* params, int32_t n_nu, JshRequest* req, uint64_t* npix) {
  if (!model || !plane || !params) {
    jsh_set_error("null descriptor");
    return JSH_ERR_INVALID;
  }
  if (n_nu < 1 || n_nu > 4096) {
    jsh_set_error("n_nu must be in [1, 4096] (got %d)", n_nu);
    return JSH_ERR_INVALID;
  }
  memset(req, 0, sizeof(*req));
  int st = jsh_compile_model(model, &req->model);
  if (st) return st;
  st = jsh_compile_plane(plane, &req->plane);
  if (st) return st;
  const jsh_params& P = *params;
  if (P.n < 1 || !(P.tau_max > 0) || !std::isfinite(P.tau_max) || !(P.tau_precision > 0) || !(P.atol >= 0) ||
      !(P.rtol >= 0) || !(P.tau_atol >= 0) || !(P.tau_rtol >= 0) || (P.atol == 0 && P.rtol == 0) ||
      (P.tau_atol == 0 && P.tau_rtol == 0) || !(P.dt_max >= 0) || P.max_steps < 0) {
    jsh_set_error("invalid integration parameters");
    return JSH_ERR_INVALID;
  }
  if (P.output != JSH_OUT_I && P.output != JSH_OUT_FULL) {
    jsh_set_error("output must be JSH_OUT_I or JSH_OUT_FULL");
    return JSH_ERR_INVALID;
  }
  if (P.precision != JSH_PREC_FP64 && P.precision != JSH_PREC_MIXED) {
    jsh_set_error("precision must be JSH_PREC_FP64 or JSH_PREC_MIXED");
    return JSH_ERR_INVALID;
  }
  if (P.schedule != JSH_SCHED_STATIC && P.schedule != JSH_SCHED_PERSISTENT) {
    jsh_set_error("schedule must be JSH_SCHED_STATIC or JSH_SCHED_PERSISTENT");
    return JSH_ERR_INVALID;
  }
  if (P.output == JSH_OUT_FULL && !req->model.b_scalar && std::fabs(model->s - 2.0) < 1e-12) {
    jsh_set_error("s = 2 makes k_C_r singular (2/(s-2), src/utils.cpp:96)");
    return JSH_ERR_INVALID;
  }
  st = jsh_resolve_hull(ctx, &req->model);
  if (st) return st;
  st = jsh_resolve_cells(ctx, &req->model);
  if (st) return st;
  // gridded fields
  int gids[3] = {req->model.grid_b, req->model.grid_n, req->model.grid_v};
  for (int k = 0; k < 3; ++k) {
    if (gids[k] < 0) continue;
    if (gids[k] >= JSH_MAX_GRIDS || !ctx->grids[gids[k]].used) {
      jsh_set_error("simulation field refers to grid %d which is not uploaded", gids[k]);
      return JSH_ERR_NOT_FOUND;
    }
    req->model.grids[k] = ctx->grids[gids[k]].view;
    int nf = ctx->grids[gids[k]].view.n_fields;
    int fields[3][2] = {{req->model.fb_p, req->model.fb_phi}, {req->model.f_n, req->model.f_n},
                        {req->model.f_v, req->model.f_v}};
    if (fields[k][0] < 0 || fields[k][0] >= nf || fields[k][1] < 0 || fields[k][1] >= nf) {
      jsh_set_error("field index out of range for grid %d", gids[k]);
      return JSH_ERR_INVALID;
    }
  }
  JshParamsDev& D = req->P;
  D.n = P.n;
  D.full = (P.output == JSH_OUT_FULL);
  D.precision = P.precision;
  D.schedule = P.schedule;
  D.flags = P.flags;
  D.tau_max = P.tau_max;
  D.tau_min = P.tau_min;
  D.dt_max = P.dt_max;
  D.tau_atol = P.tau_atol;
  D.tau_rtol = P.tau_rtol;
  D.atol = P.atol;
  D.rtol = P.rtol;
  D.tau_precision = P.tau_precision;
  D.max_steps = P.max_steps > 0 ? P.max_steps : ((int64_t)1 << 22);
  req->n_nu = n_nu;
  *npix = plane->n_across * plane->n_along;
  req->npix = *npix;
  return JSH_OK;
}

extern "C" int jsh_ctx_create(int device, uint64_t hbm_budget_bytes, jsh_ctx** out) {
  if (!out) {
    jsh_set_error("null output pointer");
    return JSH_ERR_INVALID;
  }
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    jsh_set_error("no CUDA device: %s", e != cudaSuccess ? cudaGetErrorString(e) : "count is 0");
    return JSH_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) {
    jsh_set_error("device %d out of range (%d devices)", device, n);
    return JSH_ERR_INVALID;
  }
  cudaDeviceProp prop;
  JSH_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  if (prop.major * 10 + prop.minor != 103) {
    jsh_set_error("device %d is sm_%d%d; this library is built for sm_103a only", device, prop.major, prop.minor);
    return JSH_ERR_NO_DEVICE;
  }
  JSH_CUDA_TRY(cudaSetDevice(device));
  jsh_ctx* c = new jsh_ctx();
  c->device = device;
  c->num_sms = prop.multiProcessorCount;
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  c->budget = hbm_budget_bytes ? hbm_budget_bytes : (uint64_t)(0.8 * (double)free_b);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev_start) != cudaSuccess || cudaEventCreate(&c->ev_stop) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ws_ready, cudaEventDisableTiming) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->fork[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->fork[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaMallocHost((void**)&c->h_req, sizeof(JshRequest)) != cudaSuccess ||
      cudaMallocHost((void**)&c->h_fc, 4096 * sizeof(JshFreqConst)) != cudaSuccess ||
      cudaMallocHost((void**)&c->h_counters, 8 * sizeof(unsigned long long)) != cudaSuccess) {
    jsh_set_error("context creation failed: %s", cudaGetErrorString(cudaGetLastError()));
    jsh_ctx_destroy(c);
    return JSH_ERR_CUDA;
  }
  cudaEventRecord(c->ws_ready, c->stream);
  *out = c;
  return JSH_OK;
}

extern "C" void jsh_ctx_destroy(jsh_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaDeviceSynchronize();
  if (c->ws) jsh_free_device(c, c->ws, c->ws_cap);
  for (auto& g : c->grids)
    if (g.used) jsh_free_device(c, g.mem, g.bytes);
  for (auto& h : c->hulls)
    if (h.used) jsh_free_device(c, h.mem, h.bytes);
  for (auto& h : c->cells)
    if (h.used) jsh_free_device(c, h.mem, h.bytes);
  if (c->h_req) cudaFreeHost(c->h_req);
  if (c->h_fc) cudaFreeHost(c->h_fc);
  if (c->h_counters) cudaFreeHost(c->h_counters);
  if (c->ev_start) cudaEventDestroy(c->ev_start);
  if (c->ev_stop) cudaEventDestroy(c->ev_stop);
  if (c->ws_ready) cudaEventDestroy(c->ws_ready);
  for (auto& e : c->kmarks)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->fork)
    if (e) cudaEventDestroy(e);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

// context-workspace helpers, shared with the autotuner (jsh_autotune.cpp)

int ensure_workspace(jsh_ctx* ctx, size_t need) {
  if (need <= ctx->ws_cap) return JSH_OK;
  // the previous work on the workspace must be done before it is freed
  cudaEventSynchronize(ctx->ws_ready);
  if (ctx->ws) jsh_free_device(ctx, ctx->ws, ctx->ws_cap);
  ctx->ws = nullptr;
  ctx->ws_cap = 0;
  size_t cap = std::max(need, (size_t)(1u << 20));
  void* p = nullptr;
  int st = jsh_alloc_device(ctx, cap, &p);
  if (st) return st;
  ctx->ws = p;
  ctx->ws_cap = cap;
  return JSH_OK;
}

// Enqueue one request on `stream` using the context workspace.  When
// dev_out is NULL the request writes into workspace-owned planes.
int enqueue_single(jsh_ctx* ctx, const jsh_model_desc* model, const jsh_plane_desc* plane, const double* nu_hz,
                   int32_t n_nu, const jsh_params* params, cudaStream_t stream, const jsh_image* dev_out,
                   JshRequestLayout* L_out, uint64_t* npix_out) {
  if (!nu_hz || !all_finite_positive(nu_hz, n_nu)) {
    jsh_set_error("frequencies must be finite and > 0");
    return JSH_ERR_INVALID;
  }
  JshRequest req;
  uint64_t npix = 0;
  int st = jsh_prepare_request(ctx, model, plane, params, n_nu, &req, &npix);
  if (st) return st;
  JshRequestLayout L;
  jsh_request_layout(npix, plane->n_along, plane->n_across, n_nu, dev_out == nullptr, &L);
  st = ensure_workspace(ctx, L.total);
  if (st) return st;
  char* base = (char*)ctx->ws;
  jsh_bind_request(&req, base, L, dev_out == nullptr);
  if (dev_out) {
    req.tau = dev_out->tau;
    req.l = dev_out->l;
    req.I = dev_out->I;
    req.Q = dev_out->Q;
    req.U = dev_out->U;
    req.V = dev_out->V;
    req.status = dev_out->status;
  }
  // the previous user of the workspace (possibly on another stream) must finish
  JSH_CUDA_TRY(cudaStreamWaitEvent(stream, ctx->ws_ready, 0));
  // the pinned staging buffers are reused: wait for their previous copies
  JSH_CUDA_TRY(cudaEventSynchronize(ctx->ws_ready));
  if (params->precision == JSH_PREC_MIXED) {
    st = jsh_prepare_mixed(&req, nu_hz, ctx->h_fc);
    if (st) return st;
    JSH_CUDA_TRY(cudaMemcpyAsync(base + L.off_fc, ctx->h_fc, sizeof(JshFreqConst) * n_nu, cudaMemcpyHostToDevice,
                                 stream));
  }
  *ctx->h_req = req;
  JSH_CUDA_TRY(cudaMemcpyAsync(base + L.off_req, ctx->h_req, sizeof(JshRequest), cudaMemcpyHostToDevice, stream));
  JSH_CUDA_TRY(cudaMemcpyAsync(base + L.off_nu, nu_hz, sizeof(double) * n_nu, cudaMemcpyHostToDevice, stream));
  JSH_CUDA_TRY(cudaMemsetAsync(base + L.off_counters, 0, L.off_nu - L.off_counters, stream));
  const JshRequest* d_req = (const JshRequest*)(base + L.off_req);
  JSH_CUDA_TRY(jsh_launch_plane(d_req, 1, plane->n_along, stream));
  JSH_CUDA_TRY(jsh_launch_hit(d_req, 1, npix, stream));
  JshLaunchShape shape = jsh_effective_shape(ctx, params);
  shape.fused = (req.mix.helical_log && !(params->flags & JSH_FLAG_GENERAL_KERNELS)) ? 1 : 0;
  shape.marks = nullptr;
  const bool overlap = jsh_overlap_passes(params, shape, npix * (uint64_t)n_nu);
  if (overlap && shape.overlap_key <= 0) shape.overlap_key = JSH_OVERLAP_KEY;
  shape.side = overlap ? ctx->side : nullptr;
  shape.fork = overlap ? ctx->fork : nullptr;
  ctx->kmarks_set = false;
  if ((params->flags & JSH_FLAG_KERNEL_TIMES) && params->precision == JSH_PREC_MIXED &&
      params->schedule == JSH_SCHED_PERSISTENT) {
    for (auto& e : ctx->kmarks)
      if (!e) JSH_CUDA_TRY(cudaEventCreate(&e));
    shape.marks = ctx->kmarks;
    ctx->kmarks_set = true;
    ctx->kmarks_single = shape.single != 0;
  }
  JSH_CUDA_TRY(jsh_launch_transfer(d_req, 1, params->precision, params->schedule, params->output == JSH_OUT_FULL,
                                   npix * (uint64_t)n_nu, npix, shape, (unsigned int*)(base + L.off_queue),
                                   ctx->num_sms, stream));
  JSH_CUDA_TRY(cudaEventRecord(ctx->ws_ready, stream));
  ctx->last_pending = true;
  // plane (2), hit, transfer; the persistent mixed schedule adds 3 ranking
  // kernels, and its split form the tau kernel and 3 IQUV ranking kernels
  // (twice over when the passes overlap)
  ctx->last_kernels = jsh_kernels_per_request(params->precision, params->schedule, shape.single != 0, overlap);
  ctx->last_counters_off = L.off_counters;
  ctx->last_nhit_off = L.off_nhit;
  ctx->last_npix = npix;
  ctx->last_n_nu = n_nu;
  if (L_out) *L_out = L;
  if (npix_out) *npix_out = npix;
  return JSH_OK;
}

int collect_stats(jsh_ctx* ctx, jsh_stats* s) {
  if (!ctx->last_pending) {
    *s = ctx->last;
    return JSH_OK;
  }
  JSH_CUDA_TRY(cudaEventSynchronize(ctx->ws_ready));
  char* base = (char*)ctx->ws;
  unsigned long long c[4];
  uint32_t nhit = 0;
  JSH_CUDA_TRY(cudaMemcpy(c, base + ctx->last_counters_off, sizeof(c), cudaMemcpyDeviceToHost));
  JSH_CUDA_TRY(cudaMemcpy(&nhit, base + ctx->last_nhit_off, sizeof(nhit), cudaMemcpyDeviceToHost));
  jsh_stats st{};
  st.n_pixels = ctx->last_npix;
  st.n_hit_pixels = nhit;
  st.n_work_items = (uint64_t)nhit * (uint64_t)ctx->last_n_nu;
  st.rhs_evals = c[0];
  st.steps_accepted = c[1];
  st.steps_rejected = c[2];
  st.status_or = (uint32_t)c[3];
  st.kernels_launched = ctx->last_kernels;
  ctx->last = st;
  ctx->last_pending = false;
  *s = st;
  return JSH_OK;
}



extern "C" int jsh_observation_run(jsh_ctx* ctx, const jsh_model_desc* model, const jsh_plane_desc* plane,
                                   const double* nu_hz, int32_t n_nu, const jsh_params* params, jsh_image* host_out,
                                   jsh_stats* stats) {
  if (!ctx) {
    jsh_set_error("null context");
    return JSH_ERR_INVALID;
  }
  double t0 = now_ms();
  std::lock_guard<std::mutex> lk(ctx->mu);
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  JshRequestLayout L;
  uint64_t npix = 0;
  JSH_CUDA_TRY(cudaEventRecord(ctx->ev_start, ctx->stream));
  int st = enqueue_single(ctx, model, plane, nu_hz, n_nu, params, ctx->stream, nullptr, &L, &npix);
  if (st) return st;
  JSH_CUDA_TRY(cudaEventRecord(ctx->ev_stop, ctx->stream));
  if (host_out) {
    char* base = (char*)ctx->ws;
    double* planes[6] = {host_out->tau, host_out->l, host_out->I, host_out->Q, host_out->U, host_out->V};
    size_t nb = sizeof(double) * npix * (uint64_t)n_nu;
    for (int k = 0; k < 6; ++k)
      if (planes[k]) JSH_CUDA_TRY(cudaMemcpyAsync(planes[k], base + L.off_out[k], nb, cudaMemcpyDeviceToHost, ctx->stream));
    if (host_out->status)
      JSH_CUDA_TRY(cudaMemcpyAsync(host_out->status, base + L.off_out[6], sizeof(uint32_t) * npix * (uint64_t)n_nu,
                                   cudaMemcpyDeviceToHost, ctx->stream));
    JSH_CUDA_TRY(cudaEventRecord(ctx->ws_ready, ctx->stream));
  }
  JSH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  jsh_stats s{};
  st = collect_stats(ctx, &s);
  if (st) return st;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop);
  s.device_ms = ms;
  s.total_ms = now_ms() - t0;
  ctx->last = s;
  if (stats) *stats = s;
  return JSH_OK;
}

extern "C" int jsh_observation_run_device(jsh_ctx* ctx, const jsh_model_desc* model, const jsh_plane_desc* plane,
                                          const double* nu_hz, int32_t n_nu, const jsh_params* params,
                                          void* cuda_stream, jsh_image* device_out) {
  if (!ctx || !device_out) {
    jsh_set_error("null context or output");
    return JSH_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  return enqueue_single(ctx, model, plane, nu_hz, n_nu, params, (cudaStream_t)cuda_stream, device_out, nullptr,
                        nullptr);
}

extern "C" int jsh_last_stats(jsh_ctx* ctx, jsh_stats* stats) {
  if (!ctx || !stats) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  return collect_stats(ctx, stats);
}

extern "C" int jsh_plane_rays(jsh_ctx* ctx, const jsh_plane_desc* plane, double* origins, double* direction,
                              double* pixel_sizes) {
  if (!ctx || !plane) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  JshRequest req;
  memset(&req, 0, sizeof(req));
  int st = jsh_compile_plane(plane, &req.plane);
  if (st) return st;
  uint64_t npix = plane->n_across * plane->n_along;
  JshRequestLayout L;
  jsh_request_layout(0, plane->n_along, plane->n_across, 1, false, &L);
  size_t off_o = L.total, off_s = align_up(off_o + sizeof(double) * 3 * npix);
  size_t total = align_up(off_s + sizeof(double) * npix);
  st = ensure_workspace(ctx, total);
  if (st) return st;
  JSH_CUDA_TRY(cudaEventSynchronize(ctx->ws_ready));
  char* base = (char*)ctx->ws;
  jsh_bind_request(&req, base, L, false);
  *ctx->h_req = req;
  cudaStream_t s = ctx->stream;
  JSH_CUDA_TRY(cudaMemcpyAsync(base + L.off_req, ctx->h_req, sizeof(JshRequest), cudaMemcpyHostToDevice, s));
  JSH_CUDA_TRY(jsh_launch_plane((const JshRequest*)(base + L.off_req), 1, plane->n_along, s));
  JSH_CUDA_TRY(jsh_launch_plane_rays(req.plane, (double*)(base + off_o), (double*)(base + off_s), s));
  if (origins) JSH_CUDA_TRY(cudaMemcpyAsync(origins, base + off_o, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost, s));
  if (pixel_sizes)
    JSH_CUDA_TRY(cudaMemcpyAsync(pixel_sizes, base + off_s, sizeof(double) * npix, cudaMemcpyDeviceToHost, s));
  JSH_CUDA_TRY(cudaEventRecord(ctx->ws_ready, s));
  JSH_CUDA_TRY(cudaStreamSynchronize(s));
  if (direction) {
    direction[0] = req.plane.dx;
    direction[1] = req.plane.dy;
    direction[2] = req.plane.dz;
  }
  return JSH_OK;
}

extern "C" int jsh_trace_plane(jsh_ctx* ctx, const jsh_model_desc* model, const jsh_plane_desc* plane,
                               int32_t* n_seg, double* seg, uint32_t* status) {
  if (!ctx || !model || !plane) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  JshRequest req;
  memset(&req, 0, sizeof(req));
  int st = jsh_compile_model(model, &req.model);
  if (st) return st;
  st = jsh_resolve_hull(ctx, &req.model);
  if (st) return st;
  st = jsh_compile_plane(plane, &req.plane);
  if (st) return st;
  uint64_t npix = plane->n_across * plane->n_along;
  req.npix = npix;
  req.n_nu = 0;  // the hit kernel writes no output planes
  JshRequestLayout L;
  jsh_request_layout(npix, plane->n_along, plane->n_across, 1, false, &L);
  st = ensure_workspace(ctx, L.total);
  if (st) return st;
  JSH_CUDA_TRY(cudaEventSynchronize(ctx->ws_ready));
  char* base = (char*)ctx->ws;
  jsh_bind_request(&req, base, L, false);
  *ctx->h_req = req;
  cudaStream_t s = ctx->stream;
  JSH_CUDA_TRY(cudaMemcpyAsync(base + L.off_req, ctx->h_req, sizeof(JshRequest), cudaMemcpyHostToDevice, s));
  JSH_CUDA_TRY(cudaMemsetAsync(base + L.off_nhit, 0, sizeof(uint32_t), s));
  const JshRequest* d_req = (const JshRequest*)(base + L.off_req);
  JSH_CUDA_TRY(jsh_launch_plane(d_req, 1, plane->n_along, s));
  JSH_CUDA_TRY(jsh_launch_hit(d_req, 1, npix, s));
  uint32_t nhit = 0;
  JSH_CUDA_TRY(cudaMemcpyAsync(&nhit, base + L.off_nhit, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  JSH_CUDA_TRY(cudaStreamSynchronize(s));
  std::vector<JshHit> hits(nhit);
  if (nhit) JSH_CUDA_TRY(cudaMemcpy(hits.data(), base + L.off_hits, sizeof(JshHit) * nhit, cudaMemcpyDeviceToHost));
  JSH_CUDA_TRY(cudaEventRecord(ctx->ws_ready, s));
  if (n_seg) memset(n_seg, 0, sizeof(int32_t) * npix);
  if (seg) memset(seg, 0, sizeof(double) * 12 * npix);
  if (status) memset(status, 0, sizeof(uint32_t) * npix);
  for (const JshHit& h : hits) {
    if (n_seg) n_seg[h.pix] = h.nseg;
    if (status) status[h.pix] = (uint32_t)h.status | JSH_ST_HIT;
    if (seg)
      for (int k = 0; k < h.nseg; ++k)
        for (int q = 0; q < 6; ++q) seg[12 * h.pix + 6 * k + q] = h.seg[k][q];
  }
  return JSH_OK;
}

extern "C" int jsh_hit_rays(jsh_ctx* ctx, const jsh_model_desc* model, const double* origins,
                            const double* directions, int64_t n, int32_t* n_seg, double* seg, uint32_t* status) {
  if (!ctx || !model || (n > 0 && (!origins || !directions)) || n < 0) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  if (n == 0) return JSH_OK;
  std::lock_guard<std::mutex> lk(ctx->mu);
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  JshModel m;
  int st = jsh_compile_model(model, &m);
  if (st) return st;
  st = jsh_resolve_hull(ctx, &m);
  if (st) return st;
  size_t o_orig = 0, o_dir = align_up(24 * n), o_nseg = align_up(o_dir + 24 * n), o_seg = align_up(o_nseg + 4 * n),
         o_st = align_up(o_seg + 96 * n), total = align_up(o_st + 4 * n);
  st = ensure_workspace(ctx, total);
  if (st) return st;
  JSH_CUDA_TRY(cudaEventSynchronize(ctx->ws_ready));
  char* b = (char*)ctx->ws;
  cudaStream_t s = ctx->stream;
  JSH_CUDA_TRY(cudaMemcpyAsync(b + o_orig, origins, 24 * n, cudaMemcpyHostToDevice, s));
  JSH_CUDA_TRY(cudaMemcpyAsync(b + o_dir, directions, 24 * n, cudaMemcpyHostToDevice, s));
  JSH_CUDA_TRY(jsh_launch_hit_rays(m, (double*)(b + o_orig), (double*)(b + o_dir), n, (int32_t*)(b + o_nseg),
                                   (double*)(b + o_seg), (uint32_t*)(b + o_st), s));
  if (n_seg) JSH_CUDA_TRY(cudaMemcpyAsync(n_seg, b + o_nseg, 4 * n, cudaMemcpyDeviceToHost, s));
  if (seg) JSH_CUDA_TRY(cudaMemcpyAsync(seg, b + o_seg, 96 * n, cudaMemcpyDeviceToHost, s));
  if (status) JSH_CUDA_TRY(cudaMemcpyAsync(status, b + o_st, 4 * n, cudaMemcpyDeviceToHost, s));
  JSH_CUDA_TRY(cudaEventRecord(ctx->ws_ready, s));
  JSH_CUDA_TRY(cudaStreamSynchronize(s));
  return JSH_OK;
}

cudaError_t jsh_run_peaks(int num_sms, double* fp32_tflops, double* mufu_tops, double* fp64_tflops,
                          cudaStream_t stream);

extern "C" int jsh_device_peaks(jsh_ctx* ctx, double* fp32_tflops, double* mufu_tops, double* fp64_tflops) {
  if (!ctx) {
    jsh_set_error("null context");
    return JSH_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  JSH_CUDA_TRY(jsh_run_peaks(ctx->num_sms, fp32_tflops, mufu_tops, fp64_tflops, ctx->stream));
  return JSH_OK;
}

extern "C" uint64_t jsh_request_h2d_bytes(int32_t n_nu, int32_t precision) {
  if (n_nu < 0) n_nu = 0;
  uint64_t b = sizeof(JshRequest) + sizeof(double) * (uint64_t)n_nu;
  if (precision == JSH_PREC_MIXED) b += sizeof(JshFreqConst) * (uint64_t)n_nu;
  return b;
}

extern "C" void jsh_tau_panel_rule(double* x, double* wk, double* wg) {
  for (int i = 0; i < 15; ++i) {
    if (x) x[i] = jsh_gk15_x[i];
    if (wk) wk[i] = jsh_gk15_wk[i];
    if (wg) wg[i] = jsh_gk15_wg[i];
  }
}

extern "C" int jsh_last_kernel_ms(jsh_ctx* ctx, double* tau_ms, double* iquv_rank_ms, double* iquv_ms) {
  if (!ctx) {
    jsh_set_error("null context");
    return JSH_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!ctx->kmarks_set) {
    jsh_set_error("the last request was not enqueued with JSH_FLAG_KERNEL_TIMES on the mixed persistent schedule");
    return JSH_ERR_NOT_FOUND;
  }
  JSH_CUDA_TRY(cudaEventSynchronize(ctx->kmarks[3]));
  float a = 0.f, b = 0.f, c = 0.f;
  if (!ctx->kmarks_single) {
    JSH_CUDA_TRY(cudaEventElapsedTime(&a, ctx->kmarks[0], ctx->kmarks[1]));
    JSH_CUDA_TRY(cudaEventElapsedTime(&b, ctx->kmarks[1], ctx->kmarks[2]));
  }
  JSH_CUDA_TRY(cudaEventElapsedTime(&c, ctx->kmarks[2], ctx->kmarks[3]));
  if (tau_ms) *tau_ms = a;
  if (iquv_rank_ms) *iquv_rank_ms = b;
  if (iquv_ms) *iquv_ms = c;
  return JSH_OK;
}
