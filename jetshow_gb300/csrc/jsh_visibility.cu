// jsh_visibility.cu -- the visibility step after the render: the complex
// visibilities of the rendered Stokes I image at caller-given (u, v) points,
// computed on the device so the image never leaves it.
//
// Reference: JetModelZoom.ft (jetmodel.py:114-132) with FINUFFT_NUNU
// (fourier.py:40-94, a type-3 non-uniform FFT at eps 1e-6):
//   V(u, v) = exp(-2 pi i (u dx + v dy)) sum_j I_j exp(-2 pi i (u' x_j + v' y_j)),
//   (u', v') = (u, v) R(rot) = (u cos + v sin, -u sin + v cos),
// over the pixel centres x_j = -across_j / D_A, y_j = along_j / D_A (the
// "d = -pc_y" convention of JetModelZoom.calculate_grid) and the flux
// densities I_j [Jy] of get_i_image.  Here the sum is evaluated directly and
// exactly to FP32 rounding (no gridding approximation).
//
// Structure used: the across coordinate of pixel (i, j) is s_i size_j with
// s_i = (n_across - 1)/2 - i, so with a_j = -u' size_j / D_A [cycles] the
// phase of pixel (i, j) is a_j s_i + v' y_j.  Per visibility k and column j
//   sum_i w_ij e^{-2 pi i (a_j s_i + B_j)}
//     = e^{-2 pi i (a_j c + B_j)} sum_q e^{2 pi i a_j 32 q} sum_{r<32} w_{32q+r,j} e^{2 pi i a_j r},
// so the 32 row factors e^{2 pi i a r} are built once per (k, j) from 12
// accurately reduced phases (a as a compensated FP32 pair, the product's
// rounding error recovered with fma, sincospif of the fraction), and each
// pixel costs two FMAs (a real weight times a complex factor).  The block
// factors and the column factor are reduced the same way; column sums
// accumulate in FP64.  Every phase is reduced to its fractional cycle
// before sin/cos, so phases of hundreds of cycles keep ~1e-7 accuracy.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "jsh_context.h"

namespace {

constexpr int kVisThreads = 128;  // visibilities per CTA
constexpr int kColTileMax = 8;    // image columns staged in shared memory at a time (at most)
constexpr int kMaxAcross = 16384;  // rows of one staged column: 64 KB of shared memory
constexpr int kRows = 32;         // rows per inner block

struct Cf {
  float re, im;
};
__device__ __forceinline__ Cf cmul(Cf a, Cf b) {
  return Cf{fmaf(a.re, b.re, -a.im * b.im), fmaf(a.re, b.im, a.im * b.re)};
}
// exp(2 pi i f), f in cycles
__device__ __forceinline__ Cf cis_cycles(float f) {
  float s, c;
  sincospif(2.f * f, &s, &c);
  return Cf{c, s};
}
// fractional part of (ah + al) m in cycles, m a small integer held exactly
// in FP32: ah m is split exactly into p + e by fma, p - rint(p) is exact
__device__ __forceinline__ float frac_mul(float ah, float al, float m) {
  const float p = ah * m;
  const float e = fmaf(ah, m, -p);
  return (p - rintf(p)) + fmaf(al, m, e);
}

// Weights w[f][j][i] = I[f][i][j] size_j^2 jy (FP32, column-major, rows
// padded with zeros to rows_pad) and the column constants.
__global__ void vis_weights_kernel(const double* __restrict__ I, const double* __restrict__ along_size, int n_nu,
                                   int n_across, int n_along, int rows_pad, double jy, float* __restrict__ w) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t npix = (int64_t)n_across * n_along;
  if (t >= npix * n_nu) return;
  const int f = (int)(t / npix);
  const int64_t p = t - (int64_t)f * npix;
  const int i = (int)(p / n_along), j = (int)(p - (int64_t)i * n_along);
  const double s = along_size[j];
  w[((int64_t)f * n_along + j) * rows_pad + i] = (float)(I[t] * (s * s) * jy);
}

__global__ void vis_columns_kernel(const double* __restrict__ along_size, const double* __restrict__ along_center,
                                   int n_along, double rad_per_cm, double* __restrict__ colscale,
                                   double* __restrict__ ycol) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_along) return;
  colscale[j] = -along_size[j] * rad_per_cm;
  ycol[j] = along_center[j] * rad_per_cm;
}

// Partial visibilities of columns [blockIdx.y * cols, ...) for the
// visibilities of this CTA at frequency blockIdx.z.
__global__ void __launch_bounds__(kVisThreads) vis_sum_kernel(const float* __restrict__ w,
                                                              const double* __restrict__ colscale,
                                                              const double* __restrict__ ycol,
                                                              const double* __restrict__ uvr, int64_t n_uv,
                                                              int n_along, int rows_pad, double c_rows, int cols,
                                                              int col_tile, double* __restrict__ partial) {
  extern __shared__ float4 wsh[];
  const int f = blockIdx.z;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = k < n_uv;
  double up = 0.0, vp = 0.0;
  if (valid) {
    up = uvr[((int64_t)f * n_uv + k) * 2];
    vp = uvr[((int64_t)f * n_uv + k) * 2 + 1];
  }
  const int j0 = blockIdx.y * cols;
  const int j1 = min(n_along, j0 + cols);
  const int nq = rows_pad / kRows;
  double acc_re = 0.0, acc_im = 0.0;
  for (int jt = j0; jt < j1; jt += col_tile) {
    const int nt = min(col_tile, j1 - jt);
    __syncthreads();
    const float4* src = reinterpret_cast<const float4*>(w + ((int64_t)f * n_along + jt) * rows_pad);
    const int n4 = nt * rows_pad / 4;
    for (int t = threadIdx.x; t < n4; t += blockDim.x) wsh[t] = src[t];
    __syncthreads();
    for (int jj = 0; jj < nt; ++jj) {
      const int j = jt + jj;
      const double a = up * colscale[j];  // cycles per row
      const float ah = (float)a, al = (float)(a - (double)ah);
      Cf T1[8], T8[4], T[kRows];
#pragma unroll
      for (int r = 0; r < 8; ++r) T1[r] = cis_cycles(frac_mul(ah, al, (float)r));
#pragma unroll
      for (int s = 0; s < 4; ++s) T8[s] = cis_cycles(frac_mul(ah, al, (float)(8 * s)));
#pragma unroll
      for (int r = 0; r < kRows; ++r) T[r] = cmul(T8[r >> 3], T1[r & 7]);
      const float4* wc = wsh + jj * (rows_pad / 4);
      float cr = 0.f, ci = 0.f;
      for (int q = 0; q < nq; ++q) {
        float br = 0.f, bi = 0.f;
#pragma unroll
        for (int r4 = 0; r4 < kRows / 4; ++r4) {
          const float4 v = wc[q * (kRows / 4) + r4];
          br = fmaf(v.x, T[4 * r4].re, br);
          bi = fmaf(v.x, T[4 * r4].im, bi);
          br = fmaf(v.y, T[4 * r4 + 1].re, br);
          bi = fmaf(v.y, T[4 * r4 + 1].im, bi);
          br = fmaf(v.z, T[4 * r4 + 2].re, br);
          bi = fmaf(v.z, T[4 * r4 + 2].im, bi);
          br = fmaf(v.w, T[4 * r4 + 3].re, br);
          bi = fmaf(v.w, T[4 * r4 + 3].im, bi);
        }
        if (br != 0.f || bi != 0.f) {
          const Cf Z = cis_cycles(frac_mul(ah, al, (float)(kRows * q)));
          cr = fmaf(br, Z.re, fmaf(-bi, Z.im, cr));
          ci = fmaf(br, Z.im, fmaf(bi, Z.re, ci));
        }
      }
      if (cr != 0.f || ci != 0.f) {
        // column factor exp(-2 pi i (a c + B)), the phase reduced in FP64
        const double ph = fma(a, c_rows, vp * ycol[j]);
        const Cf C = cis_cycles(-(float)(ph - rint(ph)));
        acc_re += (double)fmaf(cr, C.re, -ci * C.im);
        acc_im += (double)fmaf(cr, C.im, ci * C.re);
      }
    }
  }
  if (valid) {
    double* o = partial + (((int64_t)blockIdx.y * gridDim.z + f) * n_uv + k) * 2;
    o[0] = acc_re;
    o[1] = acc_im;
  }
}

// out[f][k] = shift[f][k] * sum over column splits (in order) of the partials.
__global__ void vis_reduce_kernel(const double* __restrict__ partial, const double* __restrict__ shift, int n_split,
                                  int n_nu, int64_t n_uv, double* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n_nu * n_uv) return;
  double re = 0.0, im = 0.0;
  for (int s = 0; s < n_split; ++s) {
    re += partial[((int64_t)s * n_nu * n_uv + t) * 2];
    im += partial[((int64_t)s * n_nu * n_uv + t) * 2 + 1];
  }
  const double sr = shift[2 * t], si = shift[2 * t + 1];
  out[2 * t] = re * sr - im * si;
  out[2 * t + 1] = re * si + im * sr;
}

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

double wall_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" int jsh_observation_visibilities(jsh_ctx* ctx, const jsh_model_desc* model, const jsh_plane_desc* plane,
                                            const double* nu_hz, int32_t n_nu, const jsh_params* params,
                                            const jsh_vis_desc* vis, const double* uv, int64_t n_uv,
                                            double* vis_out, jsh_stats* stats) {
  if (!ctx || !model || !plane || !params || !vis || (n_uv > 0 && (!uv || !vis_out)) || n_uv < 0) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  if (!(vis->rad_per_cm > 0) || !std::isfinite(vis->rad_per_cm) || !std::isfinite(vis->jy_per_cgs) ||
      !std::isfinite(vis->dx) || !std::isfinite(vis->dy) || !std::isfinite(vis->rot)) {
    jsh_set_error("visibility descriptor: rad_per_cm must be finite and > 0, the others finite");
    return JSH_ERR_INVALID;
  }
  if (n_nu < 1 || n_nu > 4096 || plane->n_along > (1u << 24) || plane->n_across > (uint64_t)kMaxAcross) {
    jsh_set_error("visibilities: n_nu in [1, 4096], n_along <= 2^24 and n_across <= %d", kMaxAcross);
    return JSH_ERR_INVALID;
  }
  for (int64_t t = 0; t < 2 * n_uv * n_nu; ++t)
    if (!std::isfinite(uv[t])) {
      jsh_set_error("uv coordinates must be finite");
      return JSH_ERR_INVALID;
    }
  {
    // the row phases are reduced in FP32 pairs: a phase step per row of
    // more than ~2^21 / rows cycles (an image sampled far below its own
    // pixel scale) is rejected rather than mis-reduced
    JshPlane pl;
    int stc = jsh_compile_plane(plane, &pl);
    if (stc) return stc;
    double umax = 0.0;
    for (int64_t t = 0; t < n_uv * n_nu; ++t) umax = std::max(umax, std::hypot(uv[2 * t], uv[2 * t + 1]));
    const double smax = std::max(pl.real_start, pl.real_start * std::pow(pl.real_base, (double)plane->n_along));
    if (umax * smax * vis->rad_per_cm * (double)(plane->n_across + kRows) > 2097152.0) {
      jsh_set_error("visibilities: |uv| x pixel size x rows exceeds 2^21 cycles (image far undersampled)");
      return JSH_ERR_INVALID;
    }
  }
  const double t_start = wall_ms();
  std::lock_guard<std::mutex> lk(ctx->mu);
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  const uint64_t npix = plane->n_across * plane->n_along;
  const int n_across = (int)plane->n_across, n_along = (int)plane->n_along;
  const int rows_pad = (n_across + kRows - 1) / kRows * kRows;
  // the render's own layout, then the visibility buffers behind it
  JshRequestLayout L;
  jsh_request_layout(npix, plane->n_along, plane->n_across, n_nu, true, &L);
  const size_t o_w = up256(L.total);
  const size_t o_col = up256(o_w + sizeof(float) * (size_t)n_nu * n_along * rows_pad);
  const size_t o_y = up256(o_col + sizeof(double) * n_along);
  const size_t o_uv = up256(o_y + sizeof(double) * n_along);
  const size_t o_shift = up256(o_uv + sizeof(double) * 2 * (size_t)n_nu * n_uv);
  const size_t o_part = up256(o_shift + sizeof(double) * 2 * (size_t)n_nu * n_uv);
  const unsigned gx = (unsigned)((n_uv + kVisThreads - 1) / kVisThreads);
  // split the columns so that about 4 CTAs per SM are in flight
  int n_split = 1;
  if (gx > 0) {
    const int64_t want = 4LL * ctx->num_sms;
    n_split = (int)std::min<int64_t>(std::max<int64_t>(1, (want + gx * n_nu - 1) / (gx * (int64_t)n_nu)), n_along);
  }
  const int cols = (n_along + n_split - 1) / n_split;
  n_split = (n_along + cols - 1) / cols;
  const size_t o_out = up256(o_part + sizeof(double) * 2 * (size_t)n_split * n_nu * n_uv);
  const size_t total = up256(o_out + sizeof(double) * 2 * (size_t)n_nu * n_uv);
  int st = ensure_workspace(ctx, total);
  if (st) return st;
  cudaStream_t s = ctx->stream;
  JSH_CUDA_TRY(cudaEventRecord(ctx->ev_start, s));
  JshRequestLayout L2;
  uint64_t np2 = 0;
  st = enqueue_single(ctx, model, plane, nu_hz, n_nu, params, s, nullptr, &L2, &np2);
  if (st) return st;
  char* base = (char*)ctx->ws;
  // rotated uv and the shift phases, on the host in FP64
  std::vector<double> uvr((size_t)2 * n_nu * n_uv), sh((size_t)2 * n_nu * n_uv);
  const double cr = cos(vis->rot), sr = sin(vis->rot);
  for (int64_t t = 0; t < (int64_t)n_nu * n_uv; ++t) {
    const double u = uv[2 * t], v = uv[2 * t + 1];
    uvr[2 * t] = u * cr + v * sr;
    uvr[2 * t + 1] = -u * sr + v * cr;
    const double ph = -2.0 * JSH_PI * (u * vis->dx + v * vis->dy);
    sh[2 * t] = cos(ph);
    sh[2 * t + 1] = sin(ph);
  }
  if (n_uv > 0) {
    JSH_CUDA_TRY(cudaMemcpyAsync(base + o_uv, uvr.data(), sizeof(double) * uvr.size(), cudaMemcpyHostToDevice, s));
    JSH_CUDA_TRY(cudaMemcpyAsync(base + o_shift, sh.data(), sizeof(double) * sh.size(), cudaMemcpyHostToDevice, s));
    JSH_CUDA_TRY(cudaMemsetAsync(base + o_w, 0, sizeof(float) * (size_t)n_nu * n_along * rows_pad, s));
    const double* I = (const double*)(base + L.off_out[2]);
    const double* asz = (const double*)(base + L.off_along_size);
    const double* acn = (const double*)(base + L.off_along_center);
    const int64_t nw = (int64_t)npix * n_nu;
    vis_weights_kernel<<<(unsigned)((nw + 255) / 256), 256, 0, s>>>(I, asz, n_nu, n_across, n_along, rows_pad,
                                                                     vis->jy_per_cgs, (float*)(base + o_w));
    vis_columns_kernel<<<(unsigned)((n_along + 255) / 256), 256, 0, s>>>(asz, acn, n_along, vis->rad_per_cm,
                                                                          (double*)(base + o_col),
                                                                          (double*)(base + o_y));
    const int col_tile = std::max(1, std::min(kColTileMax, (int)((96 * 1024) / (sizeof(float) * rows_pad))));
    const size_t smem = sizeof(float) * col_tile * rows_pad;
    if (smem > 48 * 1024)
      JSH_CUDA_TRY(cudaFuncSetAttribute(vis_sum_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    vis_sum_kernel<<<dim3(gx, (unsigned)n_split, (unsigned)n_nu), kVisThreads, smem, s>>>(
        (const float*)(base + o_w), (const double*)(base + o_col), (const double*)(base + o_y),
        (const double*)(base + o_uv), n_uv, n_along, rows_pad, 0.5 * (double)(n_across - 1), cols, col_tile,
        (double*)(base + o_part));
    const int64_t nv = (int64_t)n_nu * n_uv;
    vis_reduce_kernel<<<(unsigned)((nv + 255) / 256), 256, 0, s>>>((const double*)(base + o_part),
                                                                   (const double*)(base + o_shift), n_split, n_nu,
                                                                   n_uv, (double*)(base + o_out));
    JSH_CUDA_TRY(cudaGetLastError());
  }
  JSH_CUDA_TRY(cudaEventRecord(ctx->ev_stop, s));
  if (n_uv > 0)
    JSH_CUDA_TRY(cudaMemcpyAsync(vis_out, base + o_out, sizeof(double) * 2 * (size_t)n_nu * n_uv,
                                 cudaMemcpyDeviceToHost, s));
  JSH_CUDA_TRY(cudaEventRecord(ctx->ws_ready, s));
  JSH_CUDA_TRY(cudaStreamSynchronize(s));
  jsh_stats S{};
  st = collect_stats(ctx, &S);
  if (st) return st;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop);
  S.device_ms = ms;
  S.kernels_launched += n_uv > 0 ? 4 : 0;
  S.total_ms = wall_ms() - t_start;
  ctx->last = S;
  if (stats) *stats = S;
  return JSH_OK;
}
