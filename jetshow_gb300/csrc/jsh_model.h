// jsh_model.h -- host+device POD forms of a compiled jet model and image
// plane.  The host builds them from the C-ABI descriptors (jsh_host.cpp,
// "model compile": every parameter-only transcendental -- cos of the cone
// angle, the tgamma factors, tan(pitch), Bessel I0/I1, the tangent cone of a
// ParabaloidCone -- is evaluated once on the host with the C library, as the
// reference evaluates them in its constructors / per call with the same
// arguments).  Kernels take them by value or from constant memory.
#pragma once

#include <stdint.h>

#include "../../include/jetshow_capi.h"

#define JSH_PC 3.0856775814671913e+18
#define JSH_M_E 9.10938356e-28
#define JSH_Q_E 4.80320467299766e-10
#define JSH_C 29979245800.0
#define JSH_PI 3.141592653589793238462643383279502884
#define JSH_MAS_TO_RAD 4.84813681109536e-09

#define JSH_MAX_GRIDS 16
#define JSH_MAX_CELL_SETS 16
#define JSH_MAX_SEG 2

struct JshCone {
  double ox, oy, oz;     // apex
  double dx, dy, dz;     // unit axis
  double cos_angle;
  double big_scale;
};

struct JshGrid {         // device view of an uploaded triangulated (z, r) grid
  const double* xy;      // [n][2] (z, r) in pc
  const float* xyf;      // [n][2] the same in FP32 (mixed-precision lookups)
  const float* val;      // [n][n_fields]
  const int32_t* tri;    // [n_tri][3]
  const int32_t* bstart; // [nbx*nby + 1] bucket -> triangle list offsets
  const int32_t* bitems; // triangle ids
  int64_t n, n_tri;
  int32_t n_fields, nbx, nby, pad_;
  double x0, y0, h;      // bucket grid origin and (square) cell size
  float x0f, y0f, inv_hf;
};

// Device view of an uploaded simulation hull (SimulationGeometry): the
// upper envelope R(z) of the convex hull of the (z, r) profile as vertices
// (vz[i], vR[i]), i = 0..m, z strictly increasing; the outward half-plane of
// edge e, a_e rho + b_e z <= c_e, as abc[e][3] (a_e > 0); and the n_circle
// face normals of the polygon revolved at the azimuths 2 pi j / n_circle,
// divided by cos(pi / n_circle), as g[k][2] (x, y).  A point is inside iff
// z_min <= z <= z_max and g_k . (x, y) <= R(z) for every k.
struct JshHull {
  const double* vz;
  const double* vR;
  const double* abc;
  const double* g;
  int32_t m, n_circle;
  double z_min, z_max;
};

// Device view of an uploaded random cell set (CellsRandomVectorBField): the
// cell points (cm, FP64, and pc in FP32 for the mixed path), their unit
// directions, and a uniform bucket grid over the points' box grown by a
// quarter of its size on every side whose buckets list every point that can
// be the nearest one inside them; a query outside the grid scans every cell.
struct JshCells {
  const double* p;        // [n][3] cm
  const float* pf;        // [n][3] pc
  const double* dir;      // [n][3]
  const float* dirf;      // [n][3]
  const int32_t* bstart;  // [nbx*nby*nbz + 1]
  const int32_t* bitems;  // cell ids, ascending within a bucket
  int32_t n, nbx, nby, nbz;
  double x0, y0, z0, h;   // grid origin and bucket side [cm]
  float x0f, y0f, z0f, inv_hf;  // the same in pc (FP32)
};

struct JshModel {
  // geometry
  int32_t geo_kind;
  int32_t b_kind, n_kind, v_kind;
  int32_t b_plasma, n_plasma, b_scalar, full_capable;
  double gox, goy, goz;   // geometry origin
  double gdx, gdy, gdz;   // geometry unit direction
  double big_scale, r, r0, z0;
  JshCone cone;           // Cone, or the tangent cone of a ParabaloidCone
  int32_t hull_id, pad_hull;
  JshHull hull;           // SimulationGeometry (copy of the context's view)
  // field parameters
  double bp[8], np[8], vp[8];
  // derived field constants
  double tan_pitch, bessel0, bessel1, sin_pitch, cos_pitch;
  double v_cone_oz, v_theta;
  // coefficient constants (src/utils.cpp:40-143)
  double s, gamma_min, thermal_fraction;
  double fk_i, fk_v, fe_i, fe_v, rnd_k, rnd_e;
  double kq_ratio, eq_ratio, kfr_factor, kcr_a, kcr_b;
  // log-domain constants of the mixed-precision coefficients (see
  // jsh_fields_mixed.cuh): exponents and log2 prefactors
  double lk_i, le_i, le_v, lk_cr_b;  // log2 prefactors (frequency-free parts)
  // grids used by simulation fields
  int32_t grid_b, grid_n, grid_v;
  int32_t fb_p, fb_phi, f_n, f_v;
  JshGrid grids[3];       // [0]=B grid, [1]=N grid, [2]=V grid (copies of the views)
  // random directions added to a vector B (RandomVectorBField)
  int32_t rnd_kind, cells_id;
  double rnd_frac;
  uint64_t rnd_seed;
  JshCells cells;         // JSH_RND_CELLS (copy of the context's view)
};

struct JshPlane {
  uint64_t n_across, n_along;
  double real_start, real_base;  // pyLogspace: 10^start, 10^((stop-start)/(num-1))
  double inv_sin;                // 1/sin(los)
  double dx, dy, dz;             // ray direction (Ray ctor normalisation)
  double rx, ry, rz;             // direction normalised once more (Ray re-built at tau_max)
  double* along_size;            // device [n_along]
  double* along_center;          // device [n_along]
  double* across_pos;            // device [n_across/2][n_along]
};

#ifdef __cplusplus
extern "C++" {
// Host side: compile descriptors.  Return JSH_OK or a negative status and a
// message through jsh_set_error.
int jsh_compile_model(const jsh_model_desc* d, JshModel* m);
int jsh_compile_plane(const jsh_plane_desc* d, JshPlane* p);
void jsh_set_error(const char* fmt, ...);
}
#endif
