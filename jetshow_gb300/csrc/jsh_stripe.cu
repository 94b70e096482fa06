// jsh_stripe.cu -- stripe mode: Observation::run_stripe
// (src/Observation.cpp:310-347) with integrate_tau (src/Observation.cpp:55-123)
// and Image::getStripe (src/Image.cpp:31-41), the tau-only pass along half of
// the central row that the reference's image-size search runs.
//
// One thread per stripe pixel (row n_across / 2, columns n_along / 2 ..
// n_along - 1), all FP64: the geometry hit, then per intersection a
// constant-step classical RK4 over the const-step time range [0, L] with
// dt = L / n (odeint runge_kutta4 through make_const_step_time_range: it
// steps while (t + dt) - L <= DBL_EPSILON, t = step * dt), stopped at the
// first yielded state with tau >= tau_max, whose tau is kept and whose
// later intersections are dropped; otherwise the state after the last step.
// dtau/dt = k_I does not depend on tau, so the two middle stages share one
// evaluation.  A ray that misses keeps tau = 0.
#include <cuda_runtime.h>
#include <float.h>

#include <cmath>
#include <mutex>

#include "jsh_context.h"
#include "jsh_geometry.cuh"
#include "jsh_launch.h"
#include "jsh_transfer64.cuh"

using namespace jsh;

namespace {

__global__ void __launch_bounds__(128) stripe_tau_kernel(const JshRequest* __restrict__ req, double nu,
                                                        double* __restrict__ tau_out) {
  const JshRequest& R = *req;
  const JshPlane& pl = R.plane;
  const uint64_t c0 = pl.n_along / 2;
  const uint64_t col = c0 + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= pl.n_along) return;
  Hits h;
  geo_hit(R.model, plane_origin(pl, pl.n_across / 2, col), mk(pl.dx, pl.dy, pl.dz), h);
  const D3 rd = d3(pl.dx, pl.dy, pl.dz);
  const D3 nl = rd * -1.;
  const int n = R.P.n;
  const double tau_max = R.P.tau_max;
  double bg = 0.0;
  for (int s = 0; s < h.n; ++s) {
    const D3 pin = d3(h.s[s].in.x, h.s[s].in.y, h.s[s].in.z);
    const D3 dd = d3(h.s[s].out.x, h.s[s].out.y, h.s[s].out.z) - pin;
    const double length = sq(ad(ad(ml(dd.x, dd.x), ml(dd.y, dd.y)), ml(dd.z, dd.z)));
    const double dt = length / n;
    const Path64 P{pin, rd, nl, nu};
    double x = 0.0, t = 0.0, k1, k2, k4, dum = 0.0;
    int64_t step = 0;
    bool found = (x >= tau_max);
    if (dt > 0.0) {
      const double w1 = ml(1.0 / 6.0, dt), w2 = ml(1.0 / 3.0, dt);
      while (!found && sb(ad(t, dt), length) <= DBL_EPSILON && step <= (int64_t)n + 1) {
        Rhs64<1, false>::eval(R.model, P, true, t, &dum, &k1);
        Rhs64<1, false>::eval(R.model, P, true, ad(t, ml(0.5, dt)), &dum, &k2);
        Rhs64<1, false>::eval(R.model, P, true, ad(t, dt), &dum, &k4);
        x = ad(ad(ad(ad(x, ml(w1, k1)), ml(w2, k2)), ml(w2, k2)), ml(w1, k4));
        ++step;
        t = ml((double)step, dt);
        found = (x >= tau_max);
      }
    }
    bg += x;
    if (found) break;
  }
  tau_out[col - c0] = bg;
}

}  // namespace

extern "C" int jsh_observation_run_stripe(jsh_ctx* ctx, const jsh_model_desc* model, const jsh_plane_desc* plane,
                                          double nu_hz, int32_t n, double tau_max, double* tau_host) {
  if (!ctx || !model || !plane || !tau_host) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  if (n < 1 || !(tau_max > 0) || !(nu_hz > 0) || !std::isfinite(nu_hz)) {
    jsh_set_error("stripe needs n >= 1, tau_max > 0 and a finite frequency > 0");
    return JSH_ERR_INVALID;
  }
  jsh_params P;
  jsh_params_default(&P);
  P.n = n;
  P.tau_max = tau_max;
  std::lock_guard<std::mutex> lk(ctx->mu);
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  JshRequest req;
  uint64_t npix = 0;
  int st = jsh_prepare_request(ctx, model, plane, &P, 1, &req, &npix);
  if (st) return st;
  const uint64_t count = plane->n_along - plane->n_along / 2;
  JshRequestLayout L;
  jsh_request_layout(npix, plane->n_along, plane->n_across, 1, false, &L);
  const size_t off_out = (L.total + 255) / 256 * 256;
  st = ensure_workspace(ctx, off_out + sizeof(double) * count);
  if (st) return st;
  JSH_CUDA_TRY(cudaEventSynchronize(ctx->ws_ready));
  char* base = (char*)ctx->ws;
  jsh_bind_request(&req, base, L, false);
  *ctx->h_req = req;
  cudaStream_t s = ctx->stream;
  JSH_CUDA_TRY(cudaMemcpyAsync(base + L.off_req, ctx->h_req, sizeof(JshRequest), cudaMemcpyHostToDevice, s));
  const JshRequest* d_req = (const JshRequest*)(base + L.off_req);
  JSH_CUDA_TRY(jsh_launch_plane(d_req, 1, plane->n_along, s));
  if (count > 0) {
    stripe_tau_kernel<<<(unsigned)((count + 127) / 128), 128, 0, s>>>(d_req, nu_hz, (double*)(base + off_out));
    JSH_CUDA_TRY(cudaGetLastError());
    JSH_CUDA_TRY(cudaMemcpyAsync(tau_host, base + off_out, sizeof(double) * count, cudaMemcpyDeviceToHost, s));
  }
  JSH_CUDA_TRY(cudaEventRecord(ctx->ws_ready, s));
  JSH_CUDA_TRY(cudaStreamSynchronize(s));
  return JSH_OK;
}
