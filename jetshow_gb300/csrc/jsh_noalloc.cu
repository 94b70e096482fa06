// jsh_noalloc.cu -- jsh_observation_run_noalloc: the stream-ordered render
// with every piece of device scratch (request record, counters, hit list,
// work queue, image-plane tables, frequency constants) in one file-scope
// __device__ array instead of memory from cudaMalloc.
//
// Some callers cannot allocate device memory: hosts whose framework owns the
// whole device memory pool and forbids side allocations (a fitting service
// that hands the renderer slices of its own pool), and latency-bound loops
// that cannot take the implicit device synchronisation of cudaMalloc /
// cudaFree.  They pass their own device output planes and a stream; this
// entry point allocates nothing (no cudaMalloc, cudaFree, cudaMallocHost or
// allocating library routine).
//
// The host-side inputs (the compiled request record, the frequencies and the
// mixed-precision frequency constants) travel as the parameters of one small
// staging kernel, which writes them into the array on the caller's stream
// and clears the counters, hit count, work queue and ranking buckets that
// must start at zero; nothing reads the caller's host memory after the call
// returns.
//
// The array is sized for at most JSH_NOALLOC_MAX_PIXELS pixels,
// JSH_NOALLOC_MAX_ALONG columns and JSH_NOALLOC_MAX_NU frequencies; every
// GPU that loads the library holds it (8 MiB) until the process exits.  All
// calls share it and it keeps the last call's contents, so calls whose work
// overlaps on the GPU (different streams, or another host thread) race.  The
// first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture.
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

// Host inputs of one call, passed by value to the staging kernel.
struct NoallocInputs {
  JshRequest req;
  double nu[JSH_NOALLOC_MAX_NU];
  JshFreqConst fc[JSH_NOALLOC_MAX_NU];
};
static_assert(sizeof(NoallocInputs) < 32000, "kernel parameter space");

// One CTA: copies the request record, the frequencies and their constants
// into the scratch array and zeroes [zero, zero + zero_bytes) (8-byte words).
__global__ void __launch_bounds__(256) noalloc_stage_kernel(const NoallocInputs in, int n_nu, JshRequest* d_req,
                                                            double* d_nu, JshFreqConst* d_fc, bool mixed,
                                                            unsigned long long* zero, unsigned zero_words) {
  const unsigned t = threadIdx.x;
  {
    const unsigned long long* src = (const unsigned long long*)&in.req;
    unsigned long long* dst = (unsigned long long*)d_req;
    for (unsigned i = t; i < sizeof(JshRequest) / 8; i += blockDim.x) dst[i] = src[i];
  }
  for (int i = (int)t; i < n_nu; i += (int)blockDim.x) {
    d_nu[i] = in.nu[i];
    if (mixed) d_fc[i] = in.fc[i];
  }
  for (unsigned i = t; i < zero_words; i += blockDim.x) zero[i] = 0ull;
}
static_assert(sizeof(JshRequest) % 8 == 0, "request record copied in 8-byte words");

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
  if (uses_grid(model) || model->geometry.kind == JSH_GEO_SIMULATION) {
    jsh_set_error("gridded fields and simulation hulls live in a context; the no-alloc entry point renders "
                  "analytic models only");
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

  NoallocInputs in;
  memset(&in, 0, sizeof(in));
  uint64_t np = 0;
  st = jsh_prepare_request(nullptr, model, plane, params, n_nu, &in.req, &np);
  if (st) return st;
  JshRequestLayout L;
  jsh_request_layout(npix, plane->n_along, plane->n_across, n_nu, false, &L);
  if (L.total > JSH_NOALLOC_SCRATCH_BYTES) {
    jsh_set_error("request needs %zu scratch bytes, more than the %u of the no-alloc array", L.total,
                  JSH_NOALLOC_SCRATCH_BYTES);
    return JSH_ERR_INVALID;
  }
  jsh_bind_request(&in.req, base, L, false);
  in.req.tau = device_out->tau;
  in.req.l = device_out->l;
  in.req.I = device_out->I;
  in.req.Q = device_out->Q;
  in.req.U = device_out->U;
  in.req.V = device_out->V;
  in.req.status = device_out->status;
  const bool mixed = params->precision == JSH_PREC_MIXED;
  if (mixed) {
    st = jsh_prepare_mixed(&in.req, nu_hz, in.fc);
    if (st) return st;
  }
  memcpy(in.nu, nu_hz, sizeof(double) * n_nu);
  cudaStream_t s = (cudaStream_t)cuda_stream;
  // counters, hit count, work queue and ranking buckets start at zero on
  // every call (they lie between off_counters and off_nu)
  noalloc_stage_kernel<<<1, 256, 0, s>>>(in, n_nu, (JshRequest*)(base + L.off_req), (double*)(base + L.off_nu),
                                         (JshFreqConst*)(base + L.off_fc), mixed,
                                         (unsigned long long*)(base + L.off_counters),
                                         (unsigned)((L.off_nu - L.off_counters) / 8));
  JSH_CUDA_TRY(cudaGetLastError());
  const JshRequest* d_req = (const JshRequest*)(base + L.off_req);
  JSH_CUDA_TRY(jsh_launch_plane(d_req, 1, plane->n_along, s));
  JSH_CUDA_TRY(jsh_launch_hit(d_req, 1, npix, s));
  JshLaunchShape shape = jsh_params_shape(JshLaunchShape{128, 0, 8, 0}, params);
  shape.fused = (in.req.mix.helical_log && !(params->flags & JSH_FLAG_GENERAL_KERNELS)) ? 1 : 0;
  JSH_CUDA_TRY(jsh_launch_transfer(d_req, 1, params->precision, params->schedule, params->output == JSH_OUT_FULL,
                                   npix * (uint64_t)n_nu, npix, shape, (unsigned int*)(base + L.off_queue), sms, s));
  return JSH_OK;
}
