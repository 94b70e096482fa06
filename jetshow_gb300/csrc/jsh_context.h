// jsh_context.h -- the context behind the C ABI: device, streams, the
// workspace arena of the blocking entry points, uploaded grids, tuning.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "jsh_launch.h"

#define JSH_CUDA_TRY(expr)                                                              \
  do {                                                                                  \
    cudaError_t e_ = (expr);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      jsh_set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return JSH_ERR_CUDA;                                                              \
    }                                                                                   \
  } while (0)

// A slot's `used` flag is set (release) only after its view is complete, so
// renders that read slots without the context lock (jsh_prepare_request on
// a serving thread) never see a half-written view.
struct JshGridSlot {
  std::atomic<bool> used{false};
  JshGrid view{};
  void* mem = nullptr;  // one allocation holding every array of the grid
  size_t bytes = 0;
};

struct JshCellSlot {
  std::atomic<bool> used{false};
  JshCells view{};
  void* mem = nullptr;  // one allocation holding every array of the cell set
  size_t bytes = 0;
};

struct JshHullSlot {
  std::atomic<bool> used{false};
  JshHull view{};
  void* mem = nullptr;  // one allocation holding the profile arrays
  size_t bytes = 0;
};

// Layout of one request's device memory inside an arena allocation.
struct JshRequestLayout {
  size_t off_req, off_counters, off_nhit, off_queue, off_buckets, off_iq_count, off_iq_buckets, off_nu, off_fc,
      off_along_size, off_along_center, off_across, off_hits, off_order, off_key, off_iq_items, off_iq_order,
      off_out[7];
  size_t total;
  bool own_outputs;
};

struct jsh_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr, ws_ready = nullptr;
  cudaEvent_t kmarks[4] = {nullptr, nullptr, nullptr, nullptr};  // JSH_FLAG_KERNEL_TIMES
  bool kmarks_set = false, kmarks_single = false;
  // overlapped passes of the split form: the second stream and the fork /
  // join events (created with the context)
  cudaStream_t side = nullptr;
  cudaEvent_t fork[2] = {nullptr, nullptr};
  std::mutex mu;
  uint64_t budget = 0;
  std::atomic<uint64_t> used{0};
  void* ws = nullptr;  // workspace of the blocking / device entry points
  size_t ws_cap = 0;
  JshRequest* h_req = nullptr;               // pinned staging of one request
  JshFreqConst* h_fc = nullptr;              // pinned staging of its frequency constants [4096]
  unsigned long long* h_counters = nullptr;  // pinned [8]
  JshGridSlot grids[JSH_MAX_GRIDS];
  JshHullSlot hulls[JSH_MAX_HULLS];
  JshCellSlot cells[JSH_MAX_CELL_SETS];
  bool tuned = false;
  JshLaunchShape shape{128, 0, 8, 0};
  jsh_stats last{};
  bool last_pending = false;
  size_t last_counters_off = 0, last_nhit_off = 0;
  uint64_t last_npix = 0;
  int last_n_nu = 0;
  int last_kernels = 0;
};

// Helpers shared by the C-ABI translation units.
int jsh_prepare_request(jsh_ctx* ctx, const jsh_model_desc* model, const jsh_plane_desc* plane,
                        const jsh_params* params, int32_t n_nu, JshRequest* req, uint64_t* npix);
void jsh_request_layout(uint64_t npix, uint64_t n_along, uint64_t n_across, int32_t n_nu, bool own_outputs,
                        JshRequestLayout* L);
void jsh_bind_request(JshRequest* req, char* base, const JshRequestLayout& L, bool own_outputs);
int jsh_alloc_device(jsh_ctx* ctx, size_t bytes, void** p);
// Mixed-precision constants of a prepared request: fills req->mix (except
// the device pointer fc) and fc_host[n_nu].
int jsh_prepare_mixed(JshRequest* req, const double* nu_host, JshFreqConst* fc_host);
void jsh_free_device(jsh_ctx* ctx, void* p, size_t bytes);
JshLaunchShape jsh_effective_shape(const jsh_ctx* ctx, const jsh_params* params);
// The launch knobs of `params` (block size, CTAs per SM, refill threshold,
// register-capped build) applied over the default shape `s`, clamped to the
// ranges the launchers accept; needs no context.
JshLaunchShape jsh_params_shape(JshLaunchShape s, const jsh_params* params);
// Kernels one request launches (plane, hit, ranking, transfer).
int jsh_kernels_per_request(int precision, int schedule, bool single, bool overlap = false);
// Whether a request of `items` work items runs the split form's passes
// overlapped (JSH_FLAG_OVERLAP_PASSES, or a context shape tuned to overlap
// them; large requests on the mixed persistent schedule only, never with
// JSH_FLAG_SERIAL_PASSES or the single-kernel form).
bool jsh_overlap_passes(const jsh_params* params, const JshLaunchShape& shape, uint64_t items);
// Grow the context workspace to `need` bytes (waits for its previous user).
int ensure_workspace(jsh_ctx* ctx, size_t need);
// Enqueue one request on `stream` in the context workspace; dev_out NULL
// keeps the outputs in workspace-owned planes.  Called with ctx->mu held.
int enqueue_single(jsh_ctx* ctx, const jsh_model_desc* model, const jsh_plane_desc* plane, const double* nu_hz,
                   int32_t n_nu, const jsh_params* params, cudaStream_t stream, const jsh_image* dev_out,
                   JshRequestLayout* L_out, uint64_t* npix_out);
// SimulationGeometry: copy the context's view of hull model->hull_id into
// the compiled model (JSH_ERR_NOT_FOUND for an unknown id); no-op for the
// analytic geometries.  Called with ctx->mu held.
int jsh_resolve_hull(jsh_ctx* ctx, JshModel* model);
// Random cell set: copy the context's view of model->cells_id into the
// compiled model (JSH_ERR_NOT_FOUND for an unknown id, JSH_ERR_INVALID
// without a context); no-op for other models.
int jsh_resolve_cells(jsh_ctx* ctx, JshModel* model);
// Counters of the last enqueued request (synchronises with it).
int collect_stats(jsh_ctx* ctx, jsh_stats* s);
void jsh_set_error(const char* fmt, ...);
