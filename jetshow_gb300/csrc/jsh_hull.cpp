// jsh_hull.cpp -- SimulationGeometry's hull: built once on the host from a
// (z, r) point set, uploaded as a small profile, intersected on the device
// (jsh_geometry.cuh, simulation_hit).
//
// Reference: src/main.cpp:880-897 revolves every (z, r) point of a
// simulation grid at n_circle = 36 azimuths, (r sin phi_j, r cos phi_j, z)
// with phi_j = j 2 pi / n_circle, takes CGAL::convex_hull_3 of the cloud and
// an AABB tree of its faces; SimulationGeometry::hit (src/Geometry.cpp:97-132)
// intersects the ray's LINE with the faces and keeps two points.
//
// The hull of such a cloud has a closed form, so no 3-D hull is built: its
// support function in a direction with azimuth psi and components (u_xy,
// u_z) is max_i (r_i |u_xy| c(psi) + z_i u_z), c(psi) = max_j cos(phi_j -
// psi), which is the support function of
//     { (x, y, z) : rho(x, y) <= R(z), z_min <= z <= z_max },
// rho the gauge of the regular n_circle-gon with vertices at phi_j (rho =
// max_k g_k . (x, y), g_k the face normals at (2k + 1) pi / n_circle over
// cos(pi / n_circle)) and R the upper envelope of the 2-D convex hull of
// the (z, r) points.  The profile -- R's vertices and edge half-planes --
// and the n_circle normals are all the device needs.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "jsh_context.h"
#include "jsh_model.h"

namespace {

struct HullHost {
  std::vector<double> vz, vR, abc, g;
  double z_min = 0, z_max = 0;
};

// Upper envelope of the (z, r) hull by Andrew's monotone chain over the
// points sorted by z (per z only the largest r can be on it); collinear
// vertices are dropped.  The oracle restates the same steps in C, so both
// sides hold bit-identical profiles.
int build_profile(const double* zr, int64_t n, int32_t n_circle, HullHost* H) {
  if (n < 2 || n > (int64_t)1 << 31 || n_circle < 3 || n_circle > 4096) {
    jsh_set_error("hull needs n >= 2 points and 3 <= n_circle <= 4096 (n %lld, n_circle %d)", (long long)n,
                  n_circle);
    return JSH_ERR_INVALID;
  }
  std::vector<std::pair<double, double>> p((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    const double z = zr[2 * i], r = zr[2 * i + 1];
    if (!std::isfinite(z) || !std::isfinite(r) || r < 0) {
      jsh_set_error("hull point %lld must be finite with r >= 0", (long long)i);
      return JSH_ERR_INVALID;
    }
    p[(size_t)i] = {z, r};
  }
  std::sort(p.begin(), p.end());
  std::vector<std::pair<double, double>> q;
  for (size_t i = 0; i < p.size(); ++i) {
    if (i + 1 < p.size() && p[i + 1].first == p[i].first) continue;  // keep the largest r of each z
    q.push_back(p[i]);
  }
  if (q.size() < 2) {
    jsh_set_error("hull points span a single z: the revolved hull is flat");
    return JSH_ERR_INVALID;
  }
  std::vector<std::pair<double, double>> h;
  for (const auto& c : q) {
    while (h.size() >= 2) {
      const auto& o = h[h.size() - 2];
      const auto& a = h[h.size() - 1];
      const double cr = (a.first - o.first) * (c.second - o.second) - (a.second - o.second) * (c.first - o.first);
      if (cr >= 0) h.pop_back();
      else break;
    }
    h.push_back(c);
  }
  const size_t m = h.size() - 1;
  H->vz.resize(m + 1);
  H->vR.resize(m + 1);
  for (size_t i = 0; i <= m; ++i) {
    H->vz[i] = h[i].first;
    H->vR[i] = h[i].second;
  }
  H->abc.resize(3 * m);
  for (size_t e = 0; e < m; ++e) {
    const double a = H->vz[e + 1] - H->vz[e];
    const double b = -(H->vR[e + 1] - H->vR[e]);
    H->abc[3 * e] = a;
    H->abc[3 * e + 1] = b;
    H->abc[3 * e + 2] = a * H->vR[e] + b * H->vz[e];
  }
  H->g.resize(2 * (size_t)n_circle);
  const double inv_cos = 1.0 / cos(JSH_PI / (double)n_circle);
  for (int32_t k = 0; k < n_circle; ++k) {
    const double ang = ((2.0 * k + 1.0) * JSH_PI) / (double)n_circle;
    H->g[2 * k] = sin(ang) * inv_cos;
    H->g[2 * k + 1] = cos(ang) * inv_cos;
  }
  H->z_min = H->vz[0];
  H->z_max = H->vz[m];
  return JSH_OK;
}

}  // namespace

extern "C" int jsh_hull_upload(jsh_ctx* ctx, const double* zr, int64_t n, int32_t n_circle, int32_t* hull_id) {
  if (!ctx || !zr || !hull_id) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  HullHost H;
  int st = build_profile(zr, n, n_circle, &H);
  if (st) return st;
  std::lock_guard<std::mutex> lk(ctx->mu);
  int id = -1;
  for (int k = 0; k < JSH_MAX_HULLS && id < 0; ++k)
    if (!ctx->hulls[k].used) id = k;
  if (id < 0) {
    jsh_set_error("all %d hull slots are in use", JSH_MAX_HULLS);
    return JSH_ERR_INVALID;
  }
  const size_t m = H.vz.size() - 1;
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t o_vz = 0, o_vR = al(sizeof(double) * (m + 1)), o_abc = o_vR + al(sizeof(double) * (m + 1)),
               o_g = o_abc + al(sizeof(double) * 3 * m), total = o_g + al(sizeof(double) * H.g.size());
  JSH_CUDA_TRY(cudaSetDevice(ctx->device));
  void* mem = nullptr;
  st = jsh_alloc_device(ctx, total, &mem);
  if (st) return st;
  char* base = (char*)mem;
  cudaError_t e = cudaMemcpy(base + o_vz, H.vz.data(), sizeof(double) * (m + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(base + o_vR, H.vR.data(), sizeof(double) * (m + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(base + o_abc, H.abc.data(), sizeof(double) * 3 * m, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(base + o_g, H.g.data(), sizeof(double) * H.g.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    jsh_free_device(ctx, mem, total);
    jsh_set_error("hull upload failed: %s", cudaGetErrorString(e));
    return JSH_ERR_CUDA;
  }
  JshHullSlot& S = ctx->hulls[id];
  S.mem = mem;
  S.bytes = total;
  JshHull& V = S.view;
  V.vz = (const double*)(base + o_vz);
  V.vR = (const double*)(base + o_vR);
  V.abc = (const double*)(base + o_abc);
  V.g = (const double*)(base + o_g);
  V.m = (int32_t)m;
  V.n_circle = n_circle;
  V.z_min = H.z_min;
  V.z_max = H.z_max;
  S.used.store(true, std::memory_order_release);
  *hull_id = id;
  return JSH_OK;
}

extern "C" int jsh_hull_profile(const double* zr, int64_t n, int32_t n_circle, double* vz, double* vR,
                                int32_t* m) {
  if (!zr || !vz || !vR || !m) {
    jsh_set_error("null argument");
    return JSH_ERR_INVALID;
  }
  HullHost H;
  int st = build_profile(zr, n, n_circle, &H);
  if (st) return st;
  *m = (int32_t)(H.vz.size() - 1);
  std::copy(H.vz.begin(), H.vz.end(), vz);
  std::copy(H.vR.begin(), H.vR.end(), vR);
  return JSH_OK;
}

int jsh_resolve_hull(jsh_ctx* ctx, JshModel* model) {
  if (model->geo_kind != JSH_GEO_SIMULATION) return JSH_OK;
  if (!ctx) {
    jsh_set_error("SimulationGeometry hulls live in a context; this entry point has none");
    return JSH_ERR_INVALID;
  }
  const int id = model->hull_id;
  if (id < 0 || id >= JSH_MAX_HULLS || !ctx->hulls[id].used) {
    jsh_set_error("SimulationGeometry refers to hull %d which is not uploaded", id);
    return JSH_ERR_NOT_FOUND;
  }
  model->hull = ctx->hulls[id].view;
  return JSH_OK;
}
