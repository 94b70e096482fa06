// jsh_autotune.cpp -- launch-shape search of the persistent schedule.
//
// The persistent transfer kernel's speed depends on four knobs that leave
// its results unchanged (an item's arithmetic does not depend on which lane
// or CTA runs it): the kernel build (default, or capped at 168 registers for
// more resident warps), threads per CTA, resident CTAs per SM and the refill
// threshold (idle lanes of a warp before it pulls new items from the global
// queue).  The search times the caller's request under each shape with CUDA
// events on the context stream: first a sweep over (build, block size, CTAs
// per SM) at the current refill threshold, then a sweep of the refill
// threshold at the best triple, then serial against overlapped passes of
// the split form (the deep rays' IQUV pass beside the other rays' passes)
// at the best shape.  The fastest shape becomes the context default, used
// by every later request whose params leave the knobs at 0.
//
// No counterpart in the reference, which renders on the CPU with an OpenMP
// loop over pixels (src/Observation.cpp:44-48).
#include <float.h>

#include <vector>

#include "jsh_context.h"

namespace {

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  ~Timer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

// Time one run of the request with launch shape (bs, per_sm, refill) of the
// default or the register-capped (compact) kernel build.
int time_shape(jsh_ctx* ctx, Timer& T, const jsh_model_desc* model, const jsh_plane_desc* plane,
               const double* nu_hz, int32_t n_nu, jsh_params p, int bs, int per_sm, int refill, bool compact,
               double* ms) {
  p.block_size = bs;
  p.ctas_per_sm = per_sm;
  p.refill_threshold = refill;
  if (compact) p.flags |= JSH_FLAG_COMPACT_REGS;
  else p.flags &= ~JSH_FLAG_COMPACT_REGS;
  JSH_CUDA_TRY(cudaEventRecord(T.a, ctx->stream));
  int st = enqueue_single(ctx, model, plane, nu_hz, n_nu, &p, ctx->stream, nullptr, nullptr, nullptr);
  if (st) return st;
  JSH_CUDA_TRY(cudaEventRecord(T.b, ctx->stream));
  JSH_CUDA_TRY(cudaEventSynchronize(T.b));
  float f = 0.f;
  JSH_CUDA_TRY(cudaEventElapsedTime(&f, T.a, T.b));
  *ms = f;
  return JSH_OK;
}

}  // namespace

extern "C" int jsh_autotune(jsh_ctx* ctx, const jsh_model_desc* model, const jsh_plane_desc* plane,
                            const double* nu_hz, int32_t n_nu, const jsh_params* params, jsh_tuning* best) {
  if (!ctx || !model || !plane || !nu_hz || !params || !best) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  jsh_params p = *params;
  p.schedule = JSH_SCHED_PERSISTENT;
  // the shape sweeps time serial chains; overlap is tried last
  p.flags = (p.flags | JSH_FLAG_SERIAL_PASSES) & ~JSH_FLAG_OVERLAP_PASSES;
  Timer T;
  JSH_CUDA_TRY(cudaEventCreate(&T.a));
  JSH_CUDA_TRY(cudaEventCreate(&T.b));

  // warm-up run at the current default shape (first-touch of the workspace,
  // module load)
  const JshLaunchShape cur = ctx->shape;
  double ms = 0.0;
  int st = time_shape(ctx, T, model, plane, nu_hz, n_nu, p, cur.block_size, cur.ctas_per_sm, cur.refill_threshold,
                      cur.compact != 0, &ms);
  if (st) return st;

  const bool full = p.output == JSH_OUT_FULL;
  // the register-capped build exists for the mixed kernel only
  const bool try_compact = p.precision == JSH_PREC_MIXED;
  int b_bs = cur.block_size, b_sm = cur.ctas_per_sm, b_rf = cur.refill_threshold;
  bool b_cp = cur.compact != 0;
  double b_ms = DBL_MAX;
  for (bool cp : {false, true}) {
    if (cp && !try_compact) continue;
    for (int bs : {64, 96, 128, 192, 256}) {
      const int occ = jsh_persistent_occupancy(p.precision, full, bs, cp, (p.flags & JSH_FLAG_SINGLE_KERNEL) != 0);
      if (occ < 1) continue;
      std::vector<int> per_sm = {occ};
      if (occ > 1) per_sm.push_back(occ - 1);
      if (occ > 2) per_sm.push_back(1);
      for (int k : per_sm) {
        st = time_shape(ctx, T, model, plane, nu_hz, n_nu, p, bs, k, b_rf, cp, &ms);
        if (st) return st;
        if (ms < b_ms) {
          b_ms = ms;
          b_bs = bs;
          b_sm = k;
          b_cp = cp;
        }
      }
    }
  }
  for (int rf : {1, 2, 4, 8, 16, 24, 32}) {
    if (rf == b_rf) continue;
    st = time_shape(ctx, T, model, plane, nu_hz, n_nu, p, b_bs, b_sm, rf, b_cp, &ms);
    if (st) return st;
    if (ms < b_ms) {
      b_ms = ms;
      b_rf = rf;
    }
  }
  // serial or overlapped passes (split form of the mixed schedule, requests
  // large enough to overlap); the sweeps above ran serial chains
  bool b_ov = false;
  jsh_params po = p;
  po.flags = (po.flags & ~JSH_FLAG_SERIAL_PASSES) | JSH_FLAG_OVERLAP_PASSES;
  JshLaunchShape probe = ctx->shape;
  probe.overlap_key = 0;
  uint64_t npix = (uint64_t)plane->n_across * (uint64_t)plane->n_along;
  if (jsh_overlap_passes(&po, jsh_params_shape(probe, &po), npix * (uint64_t)n_nu)) {
    st = time_shape(ctx, T, model, plane, nu_hz, n_nu, po, b_bs, b_sm, b_rf, b_cp, &ms);
    if (st) return st;
    if (ms < b_ms) {
      b_ms = ms;
      b_ov = true;
    }
  }
  ctx->shape.block_size = b_bs;
  ctx->shape.ctas_per_sm = b_sm;
  ctx->shape.refill_threshold = b_rf;
  ctx->shape.compact = b_cp ? 1 : 0;
  ctx->shape.overlap_key = b_ov ? JSH_OVERLAP_KEY : 0;
  best->block_size = b_bs;
  best->ctas_per_sm = b_sm;
  best->refill_threshold = b_rf;
  best->compact = b_cp ? 1 : 0;
  best->overlap = b_ov ? 1 : 0;
  best->ms = b_ms;
  return JSH_OK;
}
