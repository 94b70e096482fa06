// jsh_grid.cpp -- gridded (simulation) fields: host Delaunay triangulation,
// one-time upload with a uniform-bucket point-location accelerator, and
// device interpolation at host points.
//
// Reference: SimulationInterpolater (src/SimulationInterpolater.cpp:30-117)
// builds a CGAL Delaunay_triangulation_2 of the (z, r) points and, per
// query, walks to the containing face, returns nan_value for an infinite
// face, else the barycentric combination of the three vertex values.
//
// Triangulation: incremental Bowyer-Watson with ghost triangles (one ghost
// per hull edge, joined to a vertex at infinity), points inserted in
// Hilbert-curve order and located by a visibility walk from the last new
// triangle.  The predicates are exact: coordinates are mapped to a
// 2^28-step integer lattice over the bounding box and the orientation and
// in-circle determinants are evaluated in 64- and 128-bit integers.  The
// result is the Delaunay triangulation of the lattice points, which is the
// one of the input points except for quadruples that are co-circular to
// within the lattice step (about 4e-9 of the grid extent); co-circular
// quadruples get one of their two valid diagonals.  Points that coincide on
// the lattice are merged, keeping the lowest input index.  The mapping keeps
// rows of constant z or r exactly collinear (the axis r = 0, lattice rows);
// points collinear along other directions may become slivers of the size of
// the lattice step.
#include <string.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "jsh_context.h"
#include "jsh_launch.h"

namespace {

constexpr int kInf = -1;  // the vertex at infinity

struct IP {
  int64_t x, y;
};

inline int sgn128(__int128 v) { return (v > 0) - (v < 0); }

// > 0 when a, b, c turn counter-clockwise
inline int orient(const IP& a, const IP& b, const IP& c) {
  const int64_t d = (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);  // |.| < 2^58
  return (d > 0) - (d < 0);
}

// > 0 when d lies strictly inside the circle through the counter-clockwise a, b, c
inline int incircle(const IP& a, const IP& b, const IP& c, const IP& d) {
  const int64_t adx = a.x - d.x, ady = a.y - d.y, bdx = b.x - d.x, bdy = b.y - d.y, cdx = c.x - d.x,
                cdy = c.y - d.y;
  const __int128 al = (__int128)adx * adx + (__int128)ady * ady;
  const __int128 bl = (__int128)bdx * bdx + (__int128)bdy * bdy;
  const __int128 cl = (__int128)cdx * cdx + (__int128)cdy * cdy;
  const __int128 ab = (__int128)adx * bdy - (__int128)bdx * ady;
  const __int128 bc = (__int128)bdx * cdy - (__int128)cdx * bdy;
  const __int128 ca = (__int128)cdx * ady - (__int128)adx * cdy;
  return sgn128(al * bc + bl * ca + cl * ab);  // each term < 2^115
}

// d strictly inside the segment ab (a, b, d collinear)
inline bool on_open_segment(const IP& a, const IP& b, const IP& d) {
  if (a.x != b.x) return (d.x > std::min(a.x, b.x)) && (d.x < std::max(a.x, b.x));
  return (d.y > std::min(a.y, b.y)) && (d.y < std::max(a.y, b.y));
}

// Hilbert-curve index of (x, y) on a 2^16 x 2^16 grid.
uint64_t hilbert(uint32_t x, uint32_t y) {
  uint64_t d = 0;
  for (uint32_t s = 1u << 15; s > 0; s >>= 1) {
    uint32_t rx = (x & s) ? 1 : 0, ry = (y & s) ? 1 : 0;
    d += (uint64_t)s * s * ((3 * rx) ^ ry);
    if (ry == 0) {
      if (rx == 1) {
        x = s - 1 - x;
        y = s - 1 - y;
      }
      std::swap(x, y);
    }
  }
  return d;
}

struct Tri {
  int v[3];  // counter-clockwise; kInf for the vertex at infinity
  int n[3];  // n[i]: triangle across the edge opposite v[i]
  bool alive;
};

class Delaunay {
 public:
  explicit Delaunay(const std::vector<IP>& p) : P(p) {}

  // Returns false if every point is collinear.
  bool build(const std::vector<int>& order) {
    // first three non-collinear points of the insertion order
    int a = order[0], b = -1, c = -1;
    size_t ib = 0, ic = 0;
    for (size_t i = 1; i < order.size() && b < 0; ++i)
      if (P[order[i]].x != P[a].x || P[order[i]].y != P[a].y) {
        b = order[i];
        ib = i;
      }
    if (b < 0) return false;
    for (size_t i = ib + 1; i < order.size() && c < 0; ++i)
      if (orient(P[a], P[b], P[order[i]]) != 0) {
        c = order[i];
        ic = i;
      }
    if (c < 0) return false;
    if (orient(P[a], P[b], P[c]) < 0) std::swap(b, c);
    seed(a, b, c);
    for (size_t i = 1; i < order.size(); ++i) {
      if (i == ib || i == ic) continue;
      insert(order[i]);
    }
    return true;
  }

  template <class F>
  void for_each_real(F f) const {
    for (const Tri& t : T)
      if (t.alive && t.v[0] != kInf && t.v[1] != kInf && t.v[2] != kInf) f(t);
  }

 private:
  const std::vector<IP>& P;
  std::vector<Tri> T;
  std::vector<int> free_;
  int last_ = 0;
  // scratch of one insertion
  std::vector<int> cavity_, stack_;
  std::vector<char> mark_;
  struct Edge {
    int u, w, outside;
  };
  std::vector<Edge> boundary_;

  int new_tri(int a, int b, int c) {
    int id;
    if (!free_.empty()) {
      id = free_.back();
      free_.pop_back();
    } else {
      id = (int)T.size();
      T.push_back(Tri{});
      mark_.push_back(0);
    }
    T[id] = Tri{{a, b, c}, {-1, -1, -1}, true};
    return id;
  }

  static bool is_ghost(const Tri& t) { return t.v[0] == kInf || t.v[1] == kInf || t.v[2] == kInf; }

  void seed(int a, int b, int c) {
    int t0 = new_tri(a, b, c);
    int g0 = new_tri(b, a, kInf), g1 = new_tri(c, b, kInf), g2 = new_tri(a, c, kInf);
    // link every directed edge with its reverse
    std::vector<int> ids = {t0, g0, g1, g2};
    for (int i : ids)
      for (int k = 0; k < 3; ++k) {
        int u = T[i].v[(k + 1) % 3], w = T[i].v[(k + 2) % 3];
        for (int j : ids) {
          if (j == i) continue;
          for (int m = 0; m < 3; ++m)
            if (T[j].v[(m + 1) % 3] == w && T[j].v[(m + 2) % 3] == u) T[i].n[k] = j;
        }
      }
    last_ = t0;
  }

  bool conflict(const Tri& t, const IP& p) const {
    int k = -1;
    for (int i = 0; i < 3; ++i)
      if (t.v[i] == kInf) k = i;
    if (k < 0) return incircle(P[t.v[0]], P[t.v[1]], P[t.v[2]], p) > 0;
    const IP& x = P[t.v[(k + 1) % 3]];
    const IP& y = P[t.v[(k + 2) % 3]];
    int o = orient(x, y, p);
    return o > 0 || (o == 0 && on_open_segment(x, y, p));
  }

  // A triangle in conflict with p (or -1 if p duplicates a vertex).
  int locate(const IP& p) {
    int t = last_;
    if (!T[t].alive) t = 0;
    while (!T[t].alive) ++t;
    if (is_ghost(T[t])) {
      for (int i = 0; i < 3; ++i)
        if (T[t].v[i] == kInf) t = T[t].n[i];
    }
    int rot = 0;
    for (size_t guard = 0; guard < 4 * T.size() + 16; ++guard) {
      const Tri& tr = T[t];
      int next = -1;
      for (int j = 0; j < 3 && next < 0; ++j) {
        int i = (j + rot) % 3;
        if (orient(P[tr.v[(i + 1) % 3]], P[tr.v[(i + 2) % 3]], p) < 0) next = tr.n[i];
      }
      rot = (rot + 1) % 3;
      if (next < 0) {
        for (int i = 0; i < 3; ++i)
          if (P[tr.v[i]].x == p.x && P[tr.v[i]].y == p.y) return -1;
        return t;
      }
      t = next;
      if (is_ghost(T[t])) return t;
    }
    // not reached for a Delaunay triangulation; fall back to a scan
    for (size_t i = 0; i < T.size(); ++i)
      if (T[i].alive && conflict(T[i], p)) return (int)i;
    return -1;
  }

  void insert(int pi) {
    const IP& p = P[pi];
    int t0 = locate(p);
    if (t0 < 0) return;  // duplicate lattice point: merged
    // cavity: triangles in conflict, connected to t0
    cavity_.clear();
    boundary_.clear();
    stack_.assign(1, t0);
    mark_[t0] = 1;
    while (!stack_.empty()) {
      int t = stack_.back();
      stack_.pop_back();
      cavity_.push_back(t);
      for (int i = 0; i < 3; ++i) {
        int o = T[t].n[i];
        if (mark_[o] == 1) continue;
        if (mark_[o] == 0 && conflict(T[o], p)) {
          mark_[o] = 1;
          stack_.push_back(o);
        } else {
          mark_[o] = 2;  // outside: the edge opposite v[i] bounds the cavity
          boundary_.push_back(Edge{T[t].v[(i + 1) % 3], T[t].v[(i + 2) % 3], o});
        }
      }
    }
    // reset marks of the outside neighbours for the next insertion
    for (const Edge& e : boundary_) mark_[e.outside] = 0;
    for (int t : cavity_) {
      mark_[t] = 0;
      T[t].alive = false;
      free_.push_back(t);
    }
    // star of p: one triangle per boundary edge
    std::unordered_map<int, int> by_start;
    by_start.reserve(boundary_.size() * 2);
    std::vector<int> made(boundary_.size());
    for (size_t k = 0; k < boundary_.size(); ++k) {
      const Edge& e = boundary_[k];
      int nt = new_tri(e.u, e.w, pi);
      made[k] = nt;
      T[nt].n[2] = e.outside;
      Tri& O = T[e.outside];
      for (int j = 0; j < 3; ++j)
        if (O.v[(j + 1) % 3] == e.w && O.v[(j + 2) % 3] == e.u) O.n[j] = nt;
      by_start[e.u] = nt;
    }
    for (size_t k = 0; k < boundary_.size(); ++k) {
      int nt = made[k];
      int s = by_start[boundary_[k].w];  // (w, x, p): shares the edge (w, p)
      T[nt].n[0] = s;
      T[s].n[1] = nt;
    }
    last_ = made[0];
    for (int nt : made)
      if (!is_ghost(T[nt])) last_ = nt;
  }
};

}  // namespace

extern "C" int jsh_grid_triangulate(const double* xy, int64_t n, int32_t* tri_out, int64_t* n_tri) {
  if (!xy || !tri_out || !n_tri) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  *n_tri = 0;
  if (n < 3 || n > (1 << 30)) {
    jsh_set_error("triangulation needs 3 to 2^30 points (got %lld)", (long long)n);
    return JSH_ERR_INVALID;
  }
  double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
  for (int64_t i = 0; i < n; ++i) {
    const double x = xy[2 * i], y = xy[2 * i + 1];
    if (!std::isfinite(x) || !std::isfinite(y)) {
      jsh_set_error("point %lld is not finite", (long long)i);
      return JSH_ERR_INVALID;
    }
    x0 = std::min(x0, x);
    x1 = std::max(x1, x);
    y0 = std::min(y0, y);
    y1 = std::max(y1, y);
  }
  const double ext = std::max(x1 - x0, y1 - y0);
  if (!(ext > 0)) {
    jsh_set_error("all points coincide");
    return JSH_ERR_INVALID;
  }
  const double scale = (double)((1 << 28) - 1) / ext;
  std::vector<IP> P((size_t)n);
  for (int64_t i = 0; i < n; ++i)
    P[i] = IP{(int64_t)std::llround((xy[2 * i] - x0) * scale), (int64_t)std::llround((xy[2 * i + 1] - y0) * scale)};
  // insertion order: Hilbert index, ties by input index (so of coinciding
  // lattice points the lowest index is inserted first and kept)
  std::vector<uint64_t> key((size_t)n);
  for (int64_t i = 0; i < n; ++i) key[i] = hilbert((uint32_t)(P[i].x >> 12), (uint32_t)(P[i].y >> 12));
  std::vector<int> order((size_t)n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
  // coinciding points: keep the lowest input index as the first inserted
  {
    std::unordered_map<uint64_t, int> first;
    first.reserve((size_t)n * 2);
    for (int64_t i = 0; i < n; ++i) {
      uint64_t k = ((uint64_t)P[i].x << 32) | (uint64_t)P[i].y;
      auto it = first.find(k);
      if (it == first.end()) first.emplace(k, (int)i);
    }
    std::vector<int> kept;
    kept.reserve((size_t)n);
    for (int i : order) {
      uint64_t k = ((uint64_t)P[i].x << 32) | (uint64_t)P[i].y;
      if (first[k] == i) kept.push_back(i);
    }
    order.swap(kept);
  }
  if (order.size() < 3) {
    jsh_set_error("fewer than 3 distinct points");
    return JSH_ERR_INVALID;
  }
  Delaunay D(P);
  if (!D.build(order)) {
    jsh_set_error("all points are collinear");
    return JSH_ERR_INVALID;
  }
  int64_t m = 0;
  const int64_t cap = 2 * n;
  bool over = false;
  D.for_each_real([&](const Tri& t) {
    if (m >= cap) {
      over = true;
      return;
    }
    tri_out[3 * m] = t.v[0];
    tri_out[3 * m + 1] = t.v[1];
    tri_out[3 * m + 2] = t.v[2];
    ++m;
  });
  if (over) {
    jsh_set_error("internal error: more than 2n triangles");
    return JSH_ERR_INVALID;
  }
  *n_tri = m;
  return JSH_OK;
}

// ------------------------------------------------------------- upload
extern "C" int jsh_grid_upload(jsh_ctx* ctx, const double* xy, int64_t n, const float* values, int32_t n_fields,
                               const int32_t* tri, int64_t n_tri, int32_t* grid_id) {
  if (!ctx || !xy || !values || !tri || !grid_id) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  if (n < 3 || n > (1 << 30) || n_tri < 1 || n_tri > 2 * n || n_fields < 1 || n_fields > 64) {
    jsh_set_error("invalid grid sizes (n %lld, n_tri %lld, n_fields %d)", (long long)n, (long long)n_tri, n_fields);
    return JSH_ERR_INVALID;
  }
  for (int64_t i = 0; i < 3 * n_tri; ++i)
    if (tri[i] < 0 || tri[i] >= n) {
      jsh_set_error("triangle vertex index %d out of range", tri[i]);
      return JSH_ERR_INVALID;
    }
  double x0 = xy[0], x1 = xy[0], y0 = xy[1], y1 = xy[1];
  for (int64_t i = 1; i < n; ++i) {
    x0 = std::min(x0, xy[2 * i]);
    x1 = std::max(x1, xy[2 * i]);
    y0 = std::min(y0, xy[2 * i + 1]);
    y1 = std::max(y1, xy[2 * i + 1]);
  }
  if (!std::isfinite(x0) || !std::isfinite(x1) || !std::isfinite(y0) || !std::isfinite(y1)) {
    jsh_set_error("grid points must be finite");
    return JSH_ERR_INVALID;
  }
  // square buckets, about two triangles per bucket; a triangle is listed in
  // every bucket its bounding box touches, the box grown by 1e-4 of a bucket
  // so that FP32 lookups near a bucket edge still find it
  const double ex = x1 - x0, ey = y1 - y0;
  double h = std::sqrt(std::max(ex * ey, 1e-300) / std::max(1.0, (double)n_tri / 2.0));
  if (!(h > 0) || !std::isfinite(h)) h = std::max(std::max(ex, ey), 1.0);
  h = std::max(h, std::max(ex, ey) / 65536.0);  // at most 65536 buckets per side
  const int32_t nbx = std::max(1, (int32_t)std::ceil(ex / h)), nby = std::max(1, (int32_t)std::ceil(ey / h));
  const int64_t nbk = (int64_t)nbx * nby;
  std::vector<int32_t> bstart((size_t)nbk + 1, 0);
  std::vector<int32_t> box((size_t)n_tri * 4);
  for (int64_t t = 0; t < n_tri; ++t) {
    double bx0 = INFINITY, bx1 = -INFINITY, by0 = INFINITY, by1 = -INFINITY;
    for (int k = 0; k < 3; ++k) {
      const int32_t v = tri[3 * t + k];
      bx0 = std::min(bx0, xy[2 * v]);
      bx1 = std::max(bx1, xy[2 * v]);
      by0 = std::min(by0, xy[2 * v + 1]);
      by1 = std::max(by1, xy[2 * v + 1]);
    }
    int32_t i0 = (int32_t)std::floor((bx0 - x0) / h - 1e-4), i1 = (int32_t)std::floor((bx1 - x0) / h + 1e-4);
    int32_t j0 = (int32_t)std::floor((by0 - y0) / h - 1e-4), j1 = (int32_t)std::floor((by1 - y0) / h + 1e-4);
    i0 = std::max(i0, 0);
    j0 = std::max(j0, 0);
    i1 = std::min(i1, nbx - 1);
    j1 = std::min(j1, nby - 1);
    box[4 * t] = i0, box[4 * t + 1] = i1, box[4 * t + 2] = j0, box[4 * t + 3] = j1;
    for (int32_t j = j0; j <= j1; ++j)
      for (int32_t i = i0; i <= i1; ++i) bstart[(size_t)j * nbx + i + 1]++;
  }
  for (int64_t b = 0; b < nbk; ++b) bstart[b + 1] += bstart[b];
  std::vector<int32_t> fill(bstart.begin(), bstart.end() - 1), items((size_t)bstart[nbk]);
  for (int64_t t = 0; t < n_tri; ++t)
    for (int32_t j = box[4 * t + 2]; j <= box[4 * t + 3]; ++j)
      for (int32_t i = box[4 * t]; i <= box[4 * t + 1]; ++i) items[fill[(size_t)j * nbx + i]++] = (int32_t)t;
  std::vector<float> xyf((size_t)2 * n);
  for (int64_t i = 0; i < 2 * n; ++i) xyf[i] = (float)xy[i];

  std::lock_guard<std::mutex> lk(ctx->mu);
  int id = -1;
  for (int g = 0; g < JSH_MAX_GRIDS && id < 0; ++g)
    if (!ctx->grids[g].used) id = g;
  if (id < 0) {
    jsh_set_error("all %d grid slots are in use", JSH_MAX_GRIDS);
    return JSH_ERR_INVALID;
  }
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t o_xy = 0, o_xyf = o_xy + al(sizeof(double) * 2 * n), o_val = o_xyf + al(sizeof(float) * 2 * n),
               o_tri = o_val + al(sizeof(float) * (size_t)n * n_fields), o_bs = o_tri + al(sizeof(int32_t) * 3 * n_tri),
               o_bi = o_bs + al(sizeof(int32_t) * (nbk + 1)), total = o_bi + al(sizeof(int32_t) * items.size());
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  void* mem = nullptr;
  int st = jsh_alloc_device(ctx, total, &mem);
  if (st) return st;
  char* base = (char*)mem;
  cudaError_t e = cudaMemcpy(base + o_xy, xy, sizeof(double) * 2 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(base + o_xyf, xyf.data(), sizeof(float) * 2 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(base + o_val, values, sizeof(float) * (size_t)n * n_fields, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(base + o_tri, tri, sizeof(int32_t) * 3 * n_tri, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(base + o_bs, bstart.data(), sizeof(int32_t) * (nbk + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !items.empty())
    e = cudaMemcpy(base + o_bi, items.data(), sizeof(int32_t) * items.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    jsh_free_device(ctx, mem, total);
    jsh_set_error("grid upload failed: %s", cudaGetErrorString(e));
    return JSH_ERR_CUDA;
  }
  JshGridSlot& S = ctx->grids[id];
  S.mem = mem;
  S.bytes = total;
  JshGrid& G = S.view;
  G.xy = (const double*)(base + o_xy);
  G.xyf = (const float*)(base + o_xyf);
  G.val = (const float*)(base + o_val);
  G.tri = (const int32_t*)(base + o_tri);
  G.bstart = (const int32_t*)(base + o_bs);
  G.bitems = (const int32_t*)(base + o_bi);
  G.n = n;
  G.n_tri = n_tri;
  G.n_fields = n_fields;
  G.nbx = nbx;
  G.nby = nby;
  G.x0 = x0;
  G.y0 = y0;
  G.h = h;
  G.x0f = (float)x0;
  G.y0f = (float)y0;
  G.inv_hf = (float)(1.0 / h);
  S.used.store(true, std::memory_order_release);
  *grid_id = id;
  return JSH_OK;
}

// ------------------------------------------------------------- interpolate
extern "C" int jsh_grid_interpolate(jsh_ctx* ctx, int32_t grid_id, int32_t field, const double* zr, int64_t n,
                                    double nan_value, double* out) {
  if (!ctx || (n > 0 && (!zr || !out))) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (grid_id < 0 || grid_id >= JSH_MAX_GRIDS || !ctx->grids[grid_id].used) {
    jsh_set_error("unknown grid %d", grid_id);
    return JSH_ERR_NOT_FOUND;
  }
  const JshGrid& G = ctx->grids[grid_id].view;
  if (field < 0 || field >= G.n_fields) {
    jsh_set_error("field %d out of range (grid has %d)", field, G.n_fields);
    return JSH_ERR_INVALID;
  }
  if (n <= 0) return JSH_OK;
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  const size_t in_b = (sizeof(double) * 2 * n + 255) / 256 * 256;
  int st = ensure_workspace(ctx, in_b + sizeof(double) * n);
  if (st) return st;
  char* base = (char*)ctx->ws;
  JSH_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ctx->ws_ready, 0));
  JSH_CUDA_TRY(cudaMemcpyAsync(base, zr, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, ctx->stream));
  JSH_CUDA_TRY(jsh_launch_grid_interp(G, field, (const double*)base, n, nan_value, (double*)(base + in_b), ctx->stream));
  JSH_CUDA_TRY(cudaMemcpyAsync(out, base + in_b, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  JSH_CUDA_TRY(cudaEventRecord(ctx->ws_ready, ctx->stream));
  JSH_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return JSH_OK;
}
