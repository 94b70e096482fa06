/*
 * jsh_oracle.h -- TEST INFRASTRUCTURE.  A plain-C, all-FP64 CPU restatement
 * of jetshow's per-pixel transfer path, used only as the checker of the GPU
 * library (tests, the smoke check and the CPU-baseline leg of bench.py).
 * Nothing in the product links or calls it.
 *
 * Parity status: the reference itself cannot be compiled here (it needs
 * Boost.odeint, Eigen and CGAL, none of which is installed), so this
 * restatement is pinned by (a) the reference's own golden vectors, the
 * Cone::hit cases of tests/simple_test.cpp:17-101, and (b) analytic known
 * answers of the transfer equations (see tests/test_oracle.py).  Transfer
 * parity beyond those is otherwise unpinned.
 *
 * The descriptor structs are the C-ABI's (include/jetshow_capi.h); the code
 * is independent of the product's.
 */
#ifndef JSH_ORACLE_H
#define JSH_ORACLE_H

#include "../include/jetshow_capi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct jo_counters {
  uint64_t rhs_evals;
  uint64_t steps_accepted;
  uint64_t steps_rejected;
} jo_counters;

/* Image plane rays (ImagePlane/Image/Ray constructors).  origins[npix][3],
 * direction[3], sizes[npix]; any pointer may be NULL. */
int jo_plane_rays(const jsh_plane_desc* plane, double* origins, double* direction,
                  double* sizes);

/* Hit of arbitrary rays; directions are normalised as Ray::Ray does. */
int jo_hit_rays(const jsh_model_desc* model, const double* origins,
                const double* directions, int64_t n, int32_t* n_seg, double* seg,
                uint32_t* status);

/* Render the pixels pix_idx[0..n_sel) (NULL: all pixels, n_sel ignored) of
 * the plane at n_nu frequencies.  Output planes are [n_nu][n_sel].
 * n_threads <= 0: OpenMP default.  Returns 0 or a negative status. */
int jo_render(const jsh_model_desc* model, const jsh_plane_desc* plane,
              const double* nu, int32_t n_nu, const jsh_params* params,
              const int64_t* pix_idx, int64_t n_sel, int32_t n_threads,
              jsh_image* out, jo_counters* counters);

/* Per-item RHS evaluation counts of later jo_render calls are written to
 * buf[n_nu][n_sel] when buf is not NULL (cost profiling of the workloads). */
void jo_set_item_evals(uint64_t* buf);

/* All eleven transfer coefficients at a lab-frame point for the LOS unit
 * vector n_los (pointing to the observer) and frequency nu:
 * out = {kI, kQ, kU, kV, kF, kC, hQ, etaI, etaQ, etaU, etaV}. */
int jo_coefficients(const jsh_model_desc* model, const double* point,
                    const double* n_los, double nu, double* out);

/* The field laws at a lab-frame point [cm]: out = {B (a scalar law's |B| in
 * out[0]), n, v [cm/s]}. */
int jo_fields(const jsh_model_desc* model, const double* point, double* out);

/* steps_schedule (src/utils.cpp:354-366) with the limits the I pass gives
 * it (tau_n_min 0.1, tau_n_max 100): the divisor of a segment's first step
 * by the background optical depth. */
int jo_steps_schedule(double tau, int n_min, int n_max);

/* Integrate dx/dt = a x + b (scalar) from 0 to L with the tau-pass machinery
 * (dense-output Dormand-Prince, odeint adaptive-range semantics) and return
 * x(L); used by the known-answer tests of the integrator. */
double jo_test_linear_dense(double a, double b, double L, double dt0,
                            double atol, double rtol, int64_t* n_steps);
/* Same with the controlled stepper of integrate_adaptive. */
double jo_test_linear_controlled(double a, double b, double L, double dt0,
                                 double atol, double rtol, int64_t* n_steps);
/* One Dormand-Prince step of x' = x from x=1 over h, then the dense output
 * at theta: returns dense(theta) - exp(theta*h). */
double jo_test_dense_error(double h, double theta);

/* Parsecs per mas at redshift z (NULL cosmo: the reference defaults). */
double jo_mas_to_pc(double z, const jsh_cosmology* cosmo);

/* Register a triangulated (z, r) grid under `grid_id` (0..15) for the
 * JSH_*_SIMULATION fields.  xy[n][2] in pc, values[n][n_fields]. */
int jo_grid_register(int32_t grid_id, const double* xy, int64_t n,
                     const float* values, int32_t n_fields, const int32_t* tri,
                     int64_t n_tri);
double jo_grid_value(int32_t grid_id, int32_t field, double z_pc, double r_pc,
                     double nan_value);

/* Stripe mode (Observation::run_stripe + getStripe): tau of the pixels of
 * row n_across/2, columns n_along/2 .. n_along-1, constant-step RK4 with
 * n steps per intersection, stop at tau_max.  tau_out[n_along - n_along/2]. */
int jo_stripe(const jsh_model_desc* model, const jsh_plane_desc* plane, double nu, int32_t n,
              double tau_max, double* tau_out);

/* Register the hull of SimulationGeometry under hull_id (0..15): the (z, r)
 * points zr[n][2] in pc revolved at n_circle azimuths. */
int jo_hull_register(int32_t hull_id, const double* zr, int64_t n, int32_t n_circle);
/* Vertices of a registered hull's profile R(z): vz, vR [m+1] (may be NULL). */
int jo_hull_profile(int32_t hull_id, double* vz, double* vR, int32_t* m);

/* Random vector B fields (counter-based draws, see jsh_oracle.c): the
 * Philox4x32-10 block of a counter ctr[4] and key; the random unit direction
 * of counter (k0, k1, k2) and seed; the cells of RandomCellsInSphere; a cell
 * set registered under id (0..15) for JSH_RND_CELLS; its nearest cell. */
int jo_philox4x32(const uint32_t* ctr, uint64_t key, uint32_t* out);
void jo_random_direction(uint64_t seed, uint32_t k0, uint32_t k1, uint32_t k2, double* n);
int jo_cells_generate(int64_t n, double r_min, double r_max, double theta_max, double exponent, uint64_t seed,
                      double* points, double* dirs);
int jo_cells_register(int32_t id, const double* points, const double* dirs, int64_t n);
int64_t jo_cells_nearest(int32_t id, const double* q);

int jo_openmp_threads(void);

#ifdef __cplusplus
}
#endif

#endif
