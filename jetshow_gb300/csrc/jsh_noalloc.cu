// jsh_noalloc.cu -- jsh_observation_run_noalloc: the stream-ordered render
// with every piece of device scratch (request record, counters, hit list,
// work queue, image-plane tables, frequency constants) in one file-scope
// __device__ array instead of memory from cudaMalloc.
//
// Some callers cannot allocate device memory: code that runs while a stream
// is being captured (cudaMalloc is not a stream operation and is illegal
// there), hosts whose framework owns the whole device memory pool and
// forbids side allocations, and latency-bound loops that cannot afford the
// implicit device synchronisation of cudaMalloc/cudaFree.  They pass their
// own device output planes and a stream; this entry point allocates nothing
// (no cudaMalloc, cudaFree, cudaMallocHost or allocating library routine).
//
// The array is sized for at most JSH_NOALLOC_MAX_PIXELS pixels,
// JSH_NOALLOC_MAX_ALONG columns and JSH_NOALLOC_MAX_NU frequencies; every
// GPU that loads the library holds it (8 MiB) until the process exits.  All
// calls share it and it keeps the last call's contents, so calls whose work
// overlaps on the GPU (different streams, or another process thread) race;
// the counters, hit count and queue that must start at zero are cleared by
// each call on its stream.  The first call on a device looks up the array's
// device address (cudaGetSymbolAddress) with that device current; make that
// first call before any stream capture.
#include <cuda_runtime.h>
#include <string.h>

#include <cmath>
#include <mutex>

#include "jsh_context.h"

#define JSH_NOALLOC_SCRATCH_BYTES (8u << 20)
#define JSH_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[JSH_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_setup_mu;
void* g_scratch_addr[JSH_NOALLOC_MAX_DEVICES] = {nullptr};
int g_num_sms[JSH_NOALLOC_MAX_DEVICES] = {0};

// Device address of the scratch array and the SM count of the current
// device, looked up once per device.
int setup_device(int dev, char** base, int* sms) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      jsh_set_error("cudaGetSymbolAddress of the no-alloc scratch failed: %s", cudaGetErrorString(e));
      return JSH_ERR_CUDA;
    }
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess || n <= 0) {
      jsh_set_error("cudaDeviceGetAttribute(multiprocessor count) failed: %s", cudaGetErrorString(e));
      return JSH_ERR_CUDA;
    }
    g_num_sms[dev] = n;
    g_scratch_addr[dev] = p;
  }
  *base = (char*)g_scratch_addr[dev];
  *sms = g_num_sms[dev];
  return JSH_OK;
}

bool uses_grid(const jsh_model_desc* m) {
  return m->bfield.kind == JSH_B_SIMULATION || m->nfield.kind == JSH_N_SIMULATION ||
         m->vfield.kind == JSH_V_SIMULATION;
}

}  // namespace

extern "C" int jsh_observation_run_noalloc(const jsh_model_desc* model, const jsh_plane_desc* plane,
                                           const double* nu_hz, int32_t n_nu, const jsh_params* params,
                                           void* cuda_stream, jsh_image* device_out) {
  if (!model || !plane || !nu_hz || !params || !device_out) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  if (n_nu < 1 || n_nu > JSH_NOALLOC_MAX_NU) {
    jsh_set_error("n_nu = %d outside [1, %d] of the no-alloc entry point", n_nu, JSH_NOALLOC_MAX_NU);
    return JSH_ERR_INVALID;
  }
  const uint64_t npix = plane->n_across * plane->n_along;
  if (plane->n_along > JSH_NOALLOC_MAX_ALONG || npix > JSH_NOALLOC_MAX_PIXELS) {
    jsh_set_error("image %llu x %llu exceeds the no-alloc limits (%d pixels, %d columns)",
                  (unsigned long long)plane->n_across, (unsigned long long)plane->n_along, JSH_NOALLOC_MAX_PIXELS,
                  JSH_NOALLOC_MAX_ALONG);
    return JSH_ERR_INVALID;
  }
  if (uses_grid(model)) {
    jsh_set_error("gridded fields live in a context; the no-alloc entry point renders analytic models only");
    return JSH_ERR_INVALID;
  }
  for (int i = 0; i < n_nu; ++i) {
    if (!std::isfinite(nu_hz[i]) || !(nu_hz[i] > 0)) {
      jsh_set_error("frequencies must be finite and > 0");
      return JSH_ERR_INVALID;
    }
  }
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess || dev < 0 || dev >= JSH_NOALLOC_MAX_DEVICES) {
    jsh_set_error("cudaGetDevice failed: %s", cudaGetErrorString(ce));
    return JSH_ERR_CUDA;
  }
  char* base = nullptr;
  int sms = 0;
  int st = setup_device(dev, &base, &sms);
  if (st) return st;

  JshRequest req;
  uint64_t np = 0;
  st = jsh_prepare_request(nullptr, model, plane, params, n_nu, &req, &np);
  if (st) return st;
  JshRequestLayout L;
  jsh_request_layout(npix, plane->n_along, plane->n_across, n_nu, false, &L);
  if (L.total > JSH_NOALLOC_SCRATCH_BYTES) {
    jsh_set_error("request needs %zu scratch bytes, more than the %u of the no-alloc array", L.total,
                  JSH_NOALLOC_SCRATCH_BYTES);
    return JSH_ERR_INVALID;
  }
  jsh_bind_request(&req, base, L, false);
  req.tau = device_out->tau;
  req.l = device_out->l;
  req.I = device_out->I;
  req.Q = device_out->Q;
  req.U = device_out->U;
  req.V = device_out->V;
  req.status = device_out->status;
  JshFreqConst fc[JSH_NOALLOC_MAX_NU];
  if (params->precision == JSH_PREC_MIXED) {
    st = jsh_prepare_mixed(&req, nu_hz, fc);
    if (st) return st;
  }
  cudaStream_t s = (cudaStream_t)cuda_stream;
  // host sources are pageable locals: cudaMemcpyAsync stages them before returning
  JSH_CUDA_TRY(cudaMemcpyAsync(base + L.off_req, &req, sizeof(JshRequest), cudaMemcpyHostToDevice, s));
  JSH_CUDA_TRY(cudaMemcpyAsync(base + L.off_nu, nu_hz, sizeof(double) * n_nu, cudaMemcpyHostToDevice, s));
  if (params->precision == JSH_PREC_MIXED)
    JSH_CUDA_TRY(
        cudaMemcpyAsync(base + L.off_fc, fc, sizeof(JshFreqConst) * n_nu, cudaMemcpyHostToDevice, s));
  // counters, hit count and work queue start at zero on every call
  JSH_CUDA_TRY(cudaMemsetAsync(base + L.off_counters, 0, L.off_nu - L.off_counters, s));
  const JshRequest* d_req = (const JshRequest*)(base + L.off_req);
  JSH_CUDA_TRY(jsh_launch_plane(d_req, 1, plane->n_along, s));
  JSH_CUDA_TRY(jsh_launch_hit(d_req, 1, npix, s));
  JshLaunchShape shape{params->block_size > 0 ? params->block_size : 128,
                       params->ctas_per_sm, params->refill_threshold > 0 ? params->refill_threshold : 8};
  shape.block_size = shape.block_size < 32 ? 32 : (shape.block_size > 256 ? 256 : shape.block_size / 32 * 32);
  JSH_CUDA_TRY(jsh_launch_transfer(d_req, 1, params->precision, params->schedule,
                                   params->output == JSH_OUT_FULL, npix * (uint64_t)n_nu, npix, shape,
                                   (unsigned int*)(base + L.off_queue), sms, s));
  return JSH_OK;
}
