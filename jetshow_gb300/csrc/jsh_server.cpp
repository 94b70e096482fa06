// jsh_server.cpp -- the serving loop of the C ABI: render requests of
// different image sizes and frequency counts are admitted by HBM budget,
// merged into device batches as they arrive, and run as one persistent
// transfer kernel per batch, several batches in flight on separate streams
// so that one batch's tail overlaps the next batch's bulk (continuous
// batching).  Each stream slot replays a CUDA graph of its launch sequence
// (record upload, counter reset, ray generation, hit, transfer); the graph
// is shape-independent because every kernel reads its sizes from the
// request records and the grids are sized for the slot's capacity.
//
// This replaces the reference's one-image-at-a-time Observation::run
// (src/Observation.cpp:20-41) for callers that render many models, such as
// parameter fitting (jetmodel.py:92-107) and ABC sweeps.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <thread>
#include <unordered_map>
#include <vector>

#include "jsh_context.h"

#define JSH_SERVER_MAX_NU 64

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// First-fit allocator over one device arena.
class Arena {
 public:
  void init(char* base, size_t size) {
    base_ = base;
    size_ = size;
    free_.clear();
    free_[0] = size;
  }
  bool alloc(size_t bytes, size_t* off) {
    bytes = align_up(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        size_t rest = it->second - bytes, start = it->first + bytes;
        free_.erase(it);
        if (rest) free_[start] = rest;
        used_ += bytes;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = align_up(bytes);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  char* base() const { return base_; }
  size_t size() const { return size_; }
  size_t used() const { return used_; }

 private:
  char* base_ = nullptr;
  size_t size_ = 0, used_ = 0;
  std::map<size_t, size_t> free_;
};

enum ReqState { RQ_QUEUED, RQ_RUNNING, RQ_DONE, RQ_FAILED, RQ_CANCELLED };

struct Request {
  jsh_request_id id = 0;
  ReqState state = RQ_QUEUED;
  jsh_model_desc model{};
  jsh_plane_desc plane{};
  jsh_params params{};
  std::vector<double> nu;
  JshRequest rec{};          // compiled record (device pointers filled at admission)
  JshRequestLayout L{};      // request buffers (tables, hits, outputs) inside the arena
  std::vector<JshFreqConst> fc;
  size_t arena_off = 0, arena_bytes = 0;
  uint64_t npix = 0;
  int slot = -1, slot_index = -1, batch_size = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  unsigned long long counters[4] = {0, 0, 0, 0};
  int error = JSH_OK;
  bool collecting = false;  // a jsh_server_wait is copying the result out
  char message[256] = "";
};

// Device control block of a slot: the batch's request records and the
// per-request counters / hit counts / queue, one contiguous region so one
// copy and one memset prepare a batch.
struct SlotHost {
  JshRequest recs[JSH_MAX_BATCH];
  double nu[JSH_MAX_BATCH][JSH_SERVER_MAX_NU];
  JshFreqConst fc[JSH_MAX_BATCH][JSH_SERVER_MAX_NU];
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  SlotHost* host = nullptr;  // pinned staging of the control block's upload part
  unsigned long long* h_counters = nullptr;  // pinned [JSH_MAX_BATCH][8], written by the batch's last copy
  char* dev = nullptr;       // device control block: SlotHost image + counters region
  size_t counters_off = 0, counters_bytes = 0;
  // [output kind: I-only, full Stokes][kernels: general, fused benchmark family]
  // [default kernels, Faraday-thick mode (full Stokes only; captured on first use)]
  cudaGraphExec_t graph[2][2][2] = {};
  bool busy = false;
  std::vector<Request*> batch;
  int n_req = 0;
};

}  // namespace

struct jsh_server {
  jsh_ctx* ctx = nullptr;
  jsh_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::unordered_map<jsh_request_id, std::unique_ptr<Request>> reqs;
  std::vector<Slot> slots;
  Arena arena;
  void* arena_mem = nullptr;
  size_t arena_bytes = 0;
  uint64_t next_id = 1;
  bool stop = false;
  std::thread worker;
  // capacities the slot graphs are shaped for
  uint64_t cap_pix = 0, cap_along = 0;
  int cap_nu = 0;
  cudaStream_t copy_stream = nullptr;
  std::mutex copy_mu;  // serialises result copies on copy_stream
};

namespace {

// Counters region of slot s: [JSH_MAX_BATCH][8] u64 counters, n_hit[JSH_MAX_BATCH],
// [JSH_MAX_BATCH][JSH_RANK_WORDS] ranking state, the IQUV item counts
// [JSH_MAX_BATCH][2] and their [JSH_MAX_BATCH][JSH_IQ_WORDS] ranking state,
// then the queue counters (256 bytes).
size_t nhit_off() { return align_up(sizeof(unsigned long long) * 8 * JSH_MAX_BATCH); }
size_t buckets_off() { return nhit_off() + align_up(sizeof(uint32_t) * JSH_MAX_BATCH); }
size_t iq_count_off() { return buckets_off() + align_up(sizeof(uint32_t) * JSH_RANK_WORDS * JSH_MAX_BATCH); }
size_t iq_buckets_off() { return iq_count_off() + align_up(sizeof(uint32_t) * 2 * JSH_MAX_BATCH); }
size_t counters_region_bytes() {
  return iq_buckets_off() + align_up(sizeof(uint32_t) * JSH_IQ_WORDS * JSH_MAX_BATCH) + 256;
}

// Pointers of record i into the slot's counters region.
void bind_counters(JshRequest& r, char* ctl, size_t counters_off, int i) {
  char* c = ctl + counters_off;
  r.counters = (unsigned long long*)c + 8 * i;
  r.n_hit = (uint32_t*)(c + nhit_off()) + i;
  r.buckets = (uint32_t*)(c + buckets_off()) + JSH_RANK_WORDS * i;
  r.iq_count = (uint32_t*)(c + iq_count_off()) + 2 * i;
  r.iq_buckets = (uint32_t*)(c + iq_buckets_off()) + JSH_IQ_WORDS * i;
}

int prepare_request(jsh_server* S, Request* q) {
  uint64_t npix = 0;
  int st = jsh_prepare_request(S->ctx, &q->model, &q->plane, &q->params, (int32_t)q->nu.size(), &q->rec, &npix);
  if (st) return st;
  q->npix = npix;
  jsh_request_layout(npix, q->plane.n_along, q->plane.n_across, (int32_t)q->nu.size(), true, &q->L);
  // the record, counters, n_hit, queue, nu and fc live in the slot's control
  // block; the arena block holds the tables, the hit list and the outputs
  q->arena_bytes = q->L.total - q->L.off_along_size;
  q->fc.resize(q->nu.size());
  if (q->params.precision == JSH_PREC_MIXED) {
    st = jsh_prepare_mixed(&q->rec, q->nu.data(), q->fc.data());
    if (st) return st;
  }
  return JSH_OK;
}

// Bind request q (index i of the batch in slot `sl`) to its arena block and
// the slot's control block.
void bind(jsh_server* S, Slot& sl, Request* q, int i) {
  char* blk = S->arena.base() + q->arena_off - q->L.off_along_size;  // virtual base so offsets line up
  JshRequest r = q->rec;
  jsh_bind_request(&r, blk, q->L, true);
  char* ctl = sl.dev;
  bind_counters(r, ctl, sl.counters_off, i);
  r.nu = (const double*)(ctl + offsetof(SlotHost, nu) + sizeof(double) * JSH_SERVER_MAX_NU * i);
  r.mix.fc = (const JshFreqConst*)(ctl + offsetof(SlotHost, fc) + sizeof(JshFreqConst) * JSH_SERVER_MAX_NU * i);
  sl.host->recs[i] = r;
  for (size_t f = 0; f < q->nu.size(); ++f) {
    sl.host->nu[i][f] = q->nu[f];
    sl.host->fc[i][f] = q->fc[f];
  }
}

// An empty record: zero pixels, zero frequencies (no items, no writes).
void bind_empty(Slot& sl, int i) {
  JshRequest r;
  memset(&r, 0, sizeof(r));
  bind_counters(r, sl.dev, sl.counters_off, i);
  r.plane.n_across = 2;
  r.plane.n_along = 0;
  sl.host->recs[i] = r;
}

// Enqueue (or capture) the launch sequence of slot `sl` for `n_req` records.
cudaError_t enqueue_slot(jsh_server* S, Slot& sl, int n_req, bool full, bool fused, bool ft) {
  cudaStream_t st = sl.stream;
  const JshRequest* d_recs = (const JshRequest*)sl.dev;
  cudaError_t e = cudaMemcpyAsync(sl.dev, sl.host, sizeof(SlotHost), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(sl.dev + sl.counters_off, 0, sl.counters_bytes, st);
  if (e != cudaSuccess) return e;
  e = jsh_launch_plane(d_recs, n_req, S->cap_along, st);
  if (e != cudaSuccess) return e;
  e = jsh_launch_hit(d_recs, n_req, S->cap_pix, st);
  if (e != cudaSuccess) return e;
  JshLaunchShape shape = S->ctx->shape;
  shape.fused = fused ? 1 : 0;
  shape.faraday_thick = ft ? 1 : 0;
  unsigned int* queue = (unsigned int*)(sl.dev + sl.counters_off + sl.counters_bytes - 256);
  e = jsh_launch_transfer(d_recs, n_req, S->cfg.precision, JSH_SCHED_PERSISTENT, full,
                          S->cap_pix * (uint64_t)S->cap_nu * (uint64_t)n_req, S->cap_pix, shape, queue,
                          S->ctx->num_sms, st);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(sl.h_counters, sl.dev + sl.counters_off, sizeof(unsigned long long) * 8 * JSH_MAX_BATCH,
                         cudaMemcpyDeviceToHost, st);
}

}  // namespace

namespace {

// Capture the launch sequence of slot `sl` for one output kind into a graph.
// The records are read from the control block when the graph runs, so one
// graph per (slot, output kind) serves every batch.
cudaError_t build_graph(jsh_server* S, Slot& sl, bool full, bool fused, bool ft = false) {
  cudaGraph_t g;
  cudaError_t e = cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  e = enqueue_slot(S, sl, S->cfg.max_batch_requests, full, fused, ft);
  cudaError_t e2 = cudaStreamEndCapture(sl.stream, &g);
  if (e != cudaSuccess) return e;
  if (e2 != cudaSuccess) return e2;
  e = cudaGraphInstantiate(&sl.graph[full ? 1 : 0][fused ? 1 : 0][ft ? 1 : 0], g, 0);
  cudaGraphDestroy(g);
  return e;
}

// Run one batch on slot `sl` (called with S->mu held).
int launch_batch(jsh_server* S, Slot& sl) {
  const int n = (int)sl.batch.size();
  for (int i = 0; i < n; ++i) bind(S, sl, sl.batch[i], i);
  const int cap = S->cfg.max_batch_requests;
  for (int i = n; i < cap; ++i) bind_empty(sl, i);
  const bool full = sl.batch[0]->params.output == JSH_OUT_FULL;
  // the fused kernels serve a batch whose every request is of the benchmark family
  bool fused = S->cfg.precision == JSH_PREC_MIXED;
  for (int i = 0; i < n && fused; ++i)
    fused = sl.batch[i]->rec.mix.helical_log && !(sl.batch[i]->params.flags & JSH_FLAG_GENERAL_KERNELS);
  // a batch holds requests of one kind only: with or without the
  // Faraday-thick mode (full Stokes, mixed precision)
  const bool ft = full && S->cfg.precision == JSH_PREC_MIXED &&
                  (sl.batch[0]->params.flags & JSH_FLAG_FARADAY_THICK) != 0;
  cudaError_t e = cudaSuccess;
  if (S->cfg.use_graphs) {
    cudaGraphExec_t& gx = sl.graph[full ? 1 : 0][fused ? 1 : 0][ft ? 1 : 0];
    if (!gx) e = build_graph(S, sl, full, fused, ft);  // the mode's graphs: on first use (the slot is idle)
    if (e == cudaSuccess) e = cudaGraphLaunch(gx, sl.stream);
  } else {
    e = enqueue_slot(S, sl, cap, full, fused, ft);
  }
  if (e != cudaSuccess) goto fail;
  e = cudaEventRecord(sl.done, sl.stream);
  if (e != cudaSuccess) goto fail;
  sl.busy = true;
  return JSH_OK;
fail:
  jsh_set_error("batch launch failed: %s", cudaGetErrorString(e));
  return JSH_ERR_CUDA;
}

void finish_batch(jsh_server* S, Slot& sl, bool ok) {
  const int n = (int)sl.batch.size();
  const unsigned long long* c = sl.h_counters;  // complete once the slot's done event has fired
  double t = now_ms();
  for (int i = 0; i < n; ++i) {
    Request* q = sl.batch[i];
    if (ok) {
      for (int k = 0; k < 4; ++k) q->counters[k] = c[8 * i + k];
      q->state = RQ_DONE;
    } else {
      q->state = RQ_FAILED;
      q->error = JSH_ERR_CUDA;
      snprintf(q->message, sizeof(q->message), "batch failed on the device");
    }
    q->t_done = t;
    q->batch_size = n;
  }
  sl.batch.clear();
  sl.busy = false;
}

void worker_loop(jsh_server* S) {
  cudaSetDevice(S->ctx->device);
  std::unique_lock<std::mutex> lk(S->mu);
  while (true) {
    // retire finished batches
    bool progressed = false;
    for (auto& sl : S->slots) {
      if (sl.busy) {
        cudaError_t q = cudaEventQuery(sl.done);
        if (q == cudaSuccess || (q != cudaErrorNotReady)) {
          finish_batch(S, sl, q == cudaSuccess);
          progressed = true;
        }
      }
    }
    if (progressed) S->cv_done.notify_all();
    // admit queued requests into free slots
    for (auto& sl : S->slots) {
      if (sl.busy || S->queue.empty()) continue;
      int out_kind = S->queue.front()->params.output;
      const int ft_kind = S->queue.front()->params.flags & JSH_FLAG_FARADAY_THICK;
      while (!S->queue.empty() && (int)sl.batch.size() < S->cfg.max_batch_requests) {
        Request* q = S->queue.front();
        if (q->state == RQ_CANCELLED) {
          S->queue.pop_front();
          continue;
        }
        if (q->params.output != out_kind || (q->params.flags & JSH_FLAG_FARADAY_THICK) != ft_kind) break;
        size_t off;
        if (!S->arena.alloc(q->arena_bytes, &off)) break;  // wait for memory to free up
        q->arena_off = off;
        q->state = RQ_RUNNING;
        q->t_admit = now_ms();
        sl.batch.push_back(q);
        S->queue.pop_front();
      }
      if (!sl.batch.empty()) {
        if (launch_batch(S, sl) != JSH_OK) finish_batch(S, sl, false);
        progressed = true;
      }
    }
    if (progressed) S->cv_done.notify_all();
    if (S->stop && S->queue.empty()) {
      bool any = false;
      for (auto& sl : S->slots) any |= sl.busy;
      if (!any) break;
    }
    bool busy = false;
    for (auto& sl : S->slots) busy |= sl.busy;
    if (busy) {
      // poll the in-flight batches without holding the lock
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(50));
      lk.lock();
    } else {
      S->cv_work.wait_for(lk, std::chrono::milliseconds(5));
    }
  }
}

}  // namespace

extern "C" int jsh_server_create(jsh_ctx* ctx, const jsh_server_config* cfg, jsh_server** out) {
  if (!ctx || !cfg || !out) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  *out = nullptr;
  if (cfg->max_inflight_batches < 1 || cfg->max_inflight_batches > 8 || cfg->max_batch_requests < 1 ||
      cfg->max_batch_requests > JSH_MAX_BATCH ||
      (cfg->precision != JSH_PREC_MIXED && cfg->precision != JSH_PREC_FP64)) {
    jsh_set_error("invalid server configuration");
    return JSH_ERR_INVALID;
  }
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  auto* S = new jsh_server();
  S->ctx = ctx;
  S->cfg = *cfg;
  // slot graphs are shaped for these per-request capacities
  S->cap_pix = 512 * 1024;
  S->cap_along = 4096;
  S->cap_nu = JSH_SERVER_MAX_NU;
  uint64_t budget = cfg->hbm_budget_bytes ? cfg->hbm_budget_bytes : ctx->budget / 4;
  int st = jsh_alloc_device(ctx, budget, &S->arena_mem);
  if (st) {
    delete S;
    return st;
  }
  S->arena_bytes = budget;
  S->arena.init((char*)S->arena_mem, budget);
  S->slots.resize(cfg->max_inflight_batches);
  const size_t ctl_bytes = align_up(sizeof(SlotHost)) + counters_region_bytes();
  for (auto& sl : S->slots) {
    void* dev = nullptr;
    if (jsh_alloc_device(ctx, ctl_bytes, &dev) != JSH_OK ||
        cudaMallocHost((void**)&sl.host, sizeof(SlotHost)) != cudaSuccess ||
        cudaMallocHost((void**)&sl.h_counters, sizeof(unsigned long long) * 8 * JSH_MAX_BATCH) != cudaSuccess ||
        cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
      jsh_set_error("server slot creation failed");
      S->stop = true;
      jsh_server_destroy(S);
      return JSH_ERR_CUDA;
    }
    sl.dev = (char*)dev;
    sl.counters_off = align_up(sizeof(SlotHost));
    sl.counters_bytes = counters_region_bytes();
    memset(sl.host, 0, sizeof(SlotHost));
    if (cfg->use_graphs) {
      cudaError_t e = cudaSuccess;
      for (int fk = 0; fk < 4 && e == cudaSuccess; ++fk) e = build_graph(S, sl, (fk & 1) != 0, (fk & 2) != 0);
      if (e != cudaSuccess) {
        jsh_set_error("server graph capture failed: %s", cudaGetErrorString(e));
        S->stop = true;
        jsh_server_destroy(S);
        return JSH_ERR_CUDA;
      }
    }
  }
  if (cudaStreamCreateWithFlags(&S->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
    jsh_set_error("server stream creation failed");
    S->stop = true;
    jsh_server_destroy(S);
    return JSH_ERR_CUDA;
  }
  S->worker = std::thread(worker_loop, S);
  *out = S;
  return JSH_OK;
}

extern "C" void jsh_server_destroy(jsh_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    for (auto* q : S->queue) q->state = RQ_CANCELLED;
    S->queue.clear();
  }
  S->cv_work.notify_all();
  if (S->worker.joinable()) S->worker.join();
  cudaSetDevice(S->ctx->device);
  for (auto& sl : S->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    for (auto& plane : sl.graph)
      for (auto& row : plane)
        for (auto g : row)
          if (g) cudaGraphExecDestroy(g);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.host) cudaFreeHost(sl.host);
    if (sl.h_counters) cudaFreeHost(sl.h_counters);
    if (sl.dev) jsh_free_device(S->ctx, sl.dev, align_up(sizeof(SlotHost)) + counters_region_bytes());
  }
  if (S->copy_stream) cudaStreamDestroy(S->copy_stream);
  if (S->arena_mem) jsh_free_device(S->ctx, S->arena_mem, S->arena_bytes);
  delete S;
}

extern "C" int jsh_server_submit(jsh_server* S, const jsh_model_desc* model, const jsh_plane_desc* plane,
                                 const double* nu_hz, int32_t n_nu, const jsh_params* params, jsh_request_id* id) {
  if (!S || !model || !plane || !nu_hz || !params || !id) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  if (n_nu < 1 || n_nu > JSH_SERVER_MAX_NU) {
    jsh_set_error("n_nu must be in [1, %d] for served requests", JSH_SERVER_MAX_NU);
    return JSH_ERR_INVALID;
  }
  if (plane->n_across * plane->n_along > S->cap_pix || plane->n_along > S->cap_along) {
    jsh_set_error("served images are limited to %llu pixels and %llu columns", (unsigned long long)S->cap_pix,
                  (unsigned long long)S->cap_along);
    return JSH_ERR_INVALID;
  }
  if (params->precision != S->cfg.precision) {
    jsh_set_error("request precision differs from the server's");
    return JSH_ERR_INVALID;
  }
  for (int i = 0; i < n_nu; ++i)
    if (!std::isfinite(nu_hz[i]) || !(nu_hz[i] > 0)) {
      jsh_set_error("frequencies must be finite and > 0");
      return JSH_ERR_INVALID;
    }
  auto q = std::make_unique<Request>();
  q->model = *model;
  q->plane = *plane;
  q->params = *params;
  q->params.schedule = JSH_SCHED_PERSISTENT;
  q->nu.assign(nu_hz, nu_hz + n_nu);
  q->t_submit = now_ms();
  int st = prepare_request(S, q.get());
  if (st) return st;
  if (q->arena_bytes > S->arena_bytes) {
    jsh_set_error("request needs %zu bytes, more than the server's HBM budget of %zu", q->arena_bytes,
                  S->arena_bytes);
    return JSH_ERR_OOM;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->stop) {
    jsh_set_error("server is shutting down");
    return JSH_ERR_INVALID;
  }
  q->id = S->next_id++;
  *id = q->id;
  S->queue.push_back(q.get());
  S->reqs.emplace(q->id, std::move(q));
  S->cv_work.notify_one();
  return JSH_OK;
}

extern "C" int jsh_server_poll(jsh_server* S, jsh_request_id id) {
  if (!S) return JSH_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) {
    jsh_set_error("unknown request %llu", (unsigned long long)id);
    return JSH_ERR_NOT_FOUND;
  }
  ReqState s = it->second->state;
  if (s == RQ_FAILED) return it->second->error;
  if (s == RQ_CANCELLED) return JSH_ERR_CANCELLED;
  return s == RQ_DONE ? 1 : 0;
}

extern "C" int jsh_server_wait(jsh_server* S, jsh_request_id id, int32_t timeout_ms, jsh_image* host_out,
                               jsh_request_stats* stats) {
  if (!S) return JSH_ERR_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) {
    jsh_set_error("unknown request %llu", (unsigned long long)id);
    return JSH_ERR_NOT_FOUND;
  }
  Request* q = it->second.get();
  auto ready = [&] { return q->state == RQ_DONE || q->state == RQ_FAILED || q->state == RQ_CANCELLED; };
  if (timeout_ms < 0) S->cv_done.wait(lk, ready);
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    jsh_set_error("request %llu not finished after %d ms", (unsigned long long)id, timeout_ms);
    return JSH_ERR_TIMEOUT;
  }
  if (q->collecting) {
    jsh_set_error("request %llu is already being collected", (unsigned long long)id);
    return JSH_ERR_INVALID;
  }
  q->collecting = true;
  int rc = JSH_OK;
  if (q->state == RQ_CANCELLED) rc = JSH_ERR_CANCELLED;
  if (q->state == RQ_FAILED) {
    jsh_set_error("%s", q->message);
    rc = q->error;
  }
  if (rc == JSH_OK && host_out) {
    // the block stays allocated until the release below: copy without the
    // lock so the worker keeps admitting and retiring batches meanwhile
    const char* blk = S->arena.base() + q->arena_off - q->L.off_along_size;
    const size_t n = q->npix * q->nu.size();
    const JshRequestLayout L = q->L;
    lk.unlock();
    {
      std::lock_guard<std::mutex> copy_lk(S->copy_mu);
      double* planes[6] = {host_out->tau, host_out->l, host_out->I, host_out->Q, host_out->U, host_out->V};
      for (int k = 0; k < 6 && rc == JSH_OK; ++k)
        if (planes[k] && cudaMemcpyAsync(planes[k], blk + L.off_out[k], sizeof(double) * n,
                                         cudaMemcpyDeviceToHost, S->copy_stream) != cudaSuccess)
          rc = JSH_ERR_CUDA;
      if (rc == JSH_OK && host_out->status &&
          cudaMemcpyAsync(host_out->status, blk + L.off_out[6], sizeof(uint32_t) * n, cudaMemcpyDeviceToHost,
                          S->copy_stream) != cudaSuccess)
        rc = JSH_ERR_CUDA;
      if (cudaStreamSynchronize(S->copy_stream) != cudaSuccess) rc = JSH_ERR_CUDA;
      if (rc != JSH_OK) jsh_set_error("result copy failed");
    }
    lk.lock();
  }
  double t = now_ms();
  if (stats) {
    stats->queue_ms = q->t_admit > 0 ? q->t_admit - q->t_submit : 0.0;
    stats->service_ms = q->t_admit > 0 ? t - q->t_admit : 0.0;
    stats->latency_ms = t - q->t_submit;
    stats->n_work_items = 0;
    stats->status_or = (uint32_t)q->counters[3];
    stats->batch_size = q->batch_size;
  }
  if (q->state == RQ_DONE || q->state == RQ_FAILED) S->arena.release(q->arena_off, q->arena_bytes);
  S->reqs.erase(id);
  S->cv_work.notify_one();
  return rc;
}

extern "C" int jsh_server_cancel(jsh_server* S, jsh_request_id id) {
  if (!S) return JSH_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) {
    jsh_set_error("unknown request %llu", (unsigned long long)id);
    return JSH_ERR_NOT_FOUND;
  }
  Request* q = it->second.get();
  if (q->state != RQ_QUEUED) {
    jsh_set_error("request %llu already admitted", (unsigned long long)id);
    return JSH_ERR_INVALID;
  }
  q->state = RQ_CANCELLED;
  auto qi = std::find(S->queue.begin(), S->queue.end(), q);
  if (qi != S->queue.end()) S->queue.erase(qi);
  S->cv_done.notify_all();
  return JSH_OK;
}
