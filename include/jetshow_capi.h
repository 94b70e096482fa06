/*
 * jetshow_capi.h -- C ABI of the GB300 (sm_103a) renderer for jetshow's
 * per-pixel polarised synchrotron transfer path:
 *
 *     ray -> geometry hit -> tau pass -> I / IQUV pass -> pixel value
 *
 * Plain C types only (no CUDA, no C++ and no torch types), so that a ctypes,
 * cgo, JNI or pybind11 binding can bind it directly.  Every entry point that
 * can fail returns an int status (JSH_OK == 0, negative on error) and leaves
 * a message retrievable with jsh_last_error().
 *
 * Reference interfaces replaced (paths inside the jetshow project):
 *   - Observation::run_stripe / getStripe
 *       src/Observation.cpp:310-347, src/Image.cpp:31-41 -> jsh_observation_run_stripe
 *   - Observation::run / observe_single_pixel / getImage
 *       src/Observation.cpp:20-41, src/Observation.cpp:349-395,
 *       include/Observation.h:12-24                -> jsh_observation_run
 *   - ImagePlane / Image / Ray construction
 *       src/ImagePlane.cpp:11-33, src/Image.cpp:44-194,
 *       include/logspace.h:25-33, src/Ray.cpp:9-20 -> jsh_plane_rays
 *   - BaseGeometry::hit family
 *       src/Cone.cpp:56-118, src/Cylinder.cpp:35-95,
 *       src/Parabaloid.cpp:39-60, src/ParabaloidCone.cpp:45-94
 *                                                   -> jsh_trace_plane, jsh_hit_rays
 *   - pyjetshow.get_i_image (pybind11)
 *       src/pyjetshow.cpp:69-173, :181-201         -> jsh_mas_to_pc +
 *                                                      jsh_observation_run
 *   - SimulationInterpolater / create_triangulation
 *       src/SimulationInterpolater.cpp:30-117      -> jsh_grid_triangulate,
 *                                                      jsh_grid_upload,
 *                                                      jsh_grid_interpolate
 *   - SimulationGeometry + its hull (convex_hull_3 of the revolved grid
 *     points, AABB tree of the faces)
 *       src/Geometry.cpp:92-132, src/main.cpp:880-897 -> jsh_hull_upload,
 *                                                      JSH_GEO_SIMULATION
 *   - comoving_transfer_distance2 / mas_to_pc
 *       src/utils.cpp:186-208                       -> jsh_mas_to_pc
 *   - JetModelZoom.ft + FINUFFT_NUNU.forward (type-3 NUFFT of the image)
 *       jetmodel.py:114-132, fourier.py:40-94        -> jsh_observation_visibilities
 *
 * Units follow the reference: lengths in cm, magnetic field in G, densities
 * in cm^-3, frequencies in Hz, angles in rad.  Images are row-major
 * [n_nu][n_across][n_along] doubles, the layout of Image::getImage
 * (src/Image.cpp:16-28) with a leading frequency axis.
 */
#ifndef JETSHOW_CAPI_H
#define JETSHOW_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JSH_ABI_VERSION 2 /* 2: jsh_model_desc.random */

/* ---------------------------------------------------------------- status */
#define JSH_OK 0
#define JSH_ERR_INVALID (-1)  /* bad argument or descriptor              */
#define JSH_ERR_CUDA (-2)     /* CUDA runtime error                      */
#define JSH_ERR_OOM (-3)      /* request exceeds the context HBM budget  */
#define JSH_ERR_TIMEOUT (-4)  /* wait timed out                          */
#define JSH_ERR_NOT_FOUND (-5)/* unknown request / grid id               */
#define JSH_ERR_NO_DEVICE (-6)/* no CUDA device or wrong architecture    */
#define JSH_ERR_CANCELLED (-7)/* request cancelled before it ran         */

/* Per (frequency, pixel) status bits written to jsh_image.status. */
#define JSH_ST_HIT 0x1u            /* the pixel's ray intersects the jet          */
#define JSH_ST_TAU_CROSSED 0x2u    /* tau reached tau_max; path truncated there    */
#define JSH_ST_STEP_LIMIT 0x4u     /* a segment needed more than max_steps steps   */
#define JSH_ST_FAIL_LIMIT 0x8u     /* 500 consecutive rejected steps               */
#define JSH_ST_BISECT_LIMIT 0x10u  /* tau_max crossing bisection did not converge  */
#define JSH_ST_NAN 0x20u           /* NaN/Inf met in the state or step size        */
#define JSH_ST_UB_GEOMETRY 0x40u   /* reference behaviour undefined; treated as miss */
#define JSH_ST_DT_UNDERFLOW 0x80u  /* the step no longer advances the time        */
#define JSH_ST_IQUV 0x100u         /* the I/IQUV pass ran (tau > tau_min)          */

/* ------------------------------------------------------------ geometry */
enum jsh_geometry_kind {
  JSH_GEO_CONE = 1,            /* Cone(origin, direction, angle, big_scale)        */
  JSH_GEO_CYLINDER = 2,        /* Cylinder(origin, direction, r)                   */
  JSH_GEO_PARABALOID = 3,      /* Parabaloid(origin, direction, r0, big_scale)     */
  JSH_GEO_PARABALOID_CONE = 4, /* ParabaloidCone(origin, direction, r0, z0, scale) */
  JSH_GEO_SIMULATION = 5       /* SimulationGeometry(tree): the convex hull of a
                                  revolved (z, r) point set, hull_id from
                                  jsh_hull_upload; other fields unused       */
};

typedef struct jsh_geometry_desc {
  int32_t kind;        /* enum jsh_geometry_kind */
  int32_t hull_id;     /* JSH_GEO_SIMULATION: id from jsh_hull_upload (else 0) */
  double origin[3];    /* [cm] */
  double direction[3]; /* normalised by the library, as the constructors do */
  double angle;        /* cone half-opening angle [rad] */
  double big_scale;    /* [cm] length of (half-)infinite paths (cone, paraboloid) */
  double r;            /* cylinder radius [cm] */
  double r0;           /* paraboloid radius at z = 1 pc [cm] */
  double z0;           /* ParabaloidCone break [cm] */
} jsh_geometry_desc;

/* ---------------------------------------------------------------- fields */
enum jsh_bfield_kind {
  /* scalar ("tangled") fields, src/BField.cpp:35-64 */
  JSH_B_RANDOM_SCALAR = 1,          /* p = {b0, m}:  b0 (|x|/pc)^-m              */
  JSH_B_RANDOM_SCALAR_Z = 2,        /* p = {b0, m}:  b0 (|z|/pc)^-m              */
  JSH_B_COMPOSITE_RANDOM_SCALAR_Z = 3, /* p = {b0, m_inner, m_outer, z0}          */
  /* vector fields, src/BField.cpp:67-146, :196-207 */
  JSH_B_CONST_CYLINDER = 10,        /* p = {b0, n}                               */
  JSH_B_CONST_CYLINDER_Z = 11,      /* p = {b0, n}                               */
  JSH_B_RADIAL_CONICAL = 12,        /* p = {b0, n}                               */
  JSH_B_TOROIDAL = 13,              /* p = {b0, n}    (phi = atan(y/x))          */
  JSH_B_HELICAL_CYLINDER = 14,      /* p = {b0, pitch}                           */
  JSH_B_SPIRAL_CONICAL = 15,        /* p = {b0, pitch}                           */
  JSH_B_FORCE_FREE_CYLINDRICAL = 16,/* p = {b0, mu}                              */
  /* builder-defined helical field of a conical jet (no reference class):
   * B = b0 (|x|/pc)^-n (sin(pitch) phi_hat + cos(pitch) z_hat),
   * phi_hat = (-y, x, 0)/hypot(x, y); p = {b0, n, pitch, atan_quirk}.
   * atan_quirk != 0 reproduces phi = atan(y/x) of ToroidalBField, i.e.
   * phi_hat flips sign for x < 0. */
  JSH_B_HELICAL_CONICAL = 17,
  /* gridded: p = {grid id, field index of B_p, field index of B_phi} */
  JSH_B_SIMULATION = 20
};

enum jsh_nfield_kind {
  JSH_N_CONST = 1,             /* p = {n}                                       */
  JSH_N_BK = 2,                /* p = {n0, n}:  n0 (|x|/pc)^-n                  */
  JSH_N_BKZ = 3,               /* p = {n0, n}:  n0 (|z|/pc)^-n                  */
  JSH_N_COMPOSITE_BK = 4,      /* p = {n0, n_inner, n_outer, z0}                */
  JSH_N_SIMULATION = 20        /* p = {grid id, field index}                    */
};

enum jsh_vfield_kind {
  JSH_V_CONST_FLAT = 1,              /* p = {Gamma}                              */
  JSH_V_SHEARED_FLAT = 2,            /* p = {Gamma_axis, Gamma_border, r}        */
  JSH_V_SHEATH_FLAT = 3,             /* p = {Gamma_spine, Gamma_sheath, r_sheath}*/
  JSH_V_CONST_CENTRAL = 4,           /* p = {Gamma, ox, oy, oz}                  */
  JSH_V_SHEARED_CENTRAL = 5,         /* p = {Gamma_axis, Gamma_border, theta, ox, oy, oz} */
  JSH_V_SHEATH_CENTRAL = 6,          /* p = {Gamma_spine, Gamma_sheath, theta_sheath, ox, oy, oz} */
  JSH_V_CONST_PARABOLIC = 7,         /* p = {Gamma, Rz0}                         */
  JSH_V_ACC_PARABOLIC = 8,           /* p = {Gamma0, R0, Rz0}                    */
  JSH_V_SHEARED_ACC_PARABOLIC = 9,   /* p = {Gamma_axis0, Gamma_border0, R0, Rz0}*/
  JSH_V_ACC_PARABOLIC_CONST_CONE = 10,         /* p = {Gamma0, Rz0, z0}          */
  JSH_V_SHEARED_ACC_PARABOLIC_CONST_CONE = 11, /* p = {Gamma_axis0, Gamma_border0, Rz0, z0} */
  JSH_V_SIMULATION = 20              /* p = {grid id, field index of Gamma}      */
};

typedef struct jsh_field_desc {
  int32_t kind;            /* one of the enums above */
  int32_t in_plasma_frame; /* vector B and N: 1 = given in the plasma frame */
  double p[8];             /* kind-specific parameters, see the enums */
} jsh_field_desc;

/* Random directions added to a vector B field: RandomVectorBField::bf
 * (src/BField.cpp:149-161), B(p) + fraction |B(p)| n(p) with n a unit
 * vector, the wrapper's B taken as given in the plasma frame (the wrapper
 * is constructed VectorBField(true)) whatever the wrapped field's flag.
 *  - JSH_RND_CELLS (CellsRandomVectorBField, src/BField.cpp:164-172): n is
 *    the direction of the cell nearest to p among the points of a cell set
 *    uploaded with jsh_cells_upload (RandomCells::getID, src/Cells.cpp:13-18).
 *  - JSH_RND_POINTS (PointsRandomVectorBField, src/BField.cpp:175-193): a
 *    fresh direction at every right-hand-side evaluation.  The reference
 *    draws it from a per-OpenMP-thread Mersenne Twister, so its images
 *    depend on the thread schedule; here the draw is a counter-based
 *    function of (seed, pixel, frequency, evaluation index): the same
 *    render gives the same image, alone or batched with others.
 * Directions are drawn with Philox4x32-10 (Salmon et al., SC'11) by
 * rejection from the cube [-1, 1]^3 and normalised in correctly rounded
 * FP64, so host, device and a C restatement draw the same bits. */
enum jsh_random_kind { JSH_RND_NONE = 0, JSH_RND_CELLS = 1, JSH_RND_POINTS = 2 };

typedef struct jsh_random_desc {
  int32_t kind;     /* enum jsh_random_kind */
  int32_t cells_id; /* JSH_RND_CELLS: id from jsh_cells_upload */
  double fraction;  /* rnd_fraction of the reference (>= 0) */
  uint64_t seed;    /* JSH_RND_POINTS: key of the direction stream */
} jsh_random_desc;

typedef struct jsh_model_desc {
  jsh_geometry_desc geometry;
  jsh_field_desc bfield;
  jsh_field_desc nfield;
  jsh_field_desc vfield;
  double s;                /* power-law index in the coefficients
                              (the reference hard-codes s = 3.42, src/Jet.cpp:32) */
  double gamma_min;        /* low-energy cut-off in k_F_r, k_C_r (src/utils.cpp:86-98) */
  double thermal_fraction; /* n_th / n for cold-plasma k_F_c, k_C_c terms (builder-defined) */
  jsh_random_desc random;  /* random directions added to a vector B field (kind 0: none) */
} jsh_model_desc;

/* ----------------------------------------------------------- image plane */
typedef struct jsh_plane_desc {
  uint64_t n_across;          /* image_size.first; must be even */
  uint64_t n_along;           /* image_size.second */
  double lg_pixel_size_start_cm;
  double lg_pixel_size_stop_cm;
  double los_angle;           /* [rad] */
} jsh_plane_desc;

/* ----------------------------------------------------------- parameters */
enum jsh_output { JSH_OUT_I = 1, JSH_OUT_FULL = 2 };
enum jsh_precision {
  JSH_PREC_FP64 = 1,  /* every operation in FP64 (the plain GPU drop-in)        */
  JSH_PREC_MIXED = 2  /* FP32 RHS and RK stages; FP64 tau, Faraday angle, t,
                         step-size control and error norm                       */
};
enum jsh_schedule {
  JSH_SCHED_STATIC = 1,     /* one thread per (ray, frequency) for its lifetime */
  JSH_SCHED_PERSISTENT = 2  /* persistent CTAs, global work queue, lanes refilled
                               from the queue as their rays finish              */
};

typedef struct jsh_params {
  int32_t n;               /* initial step = L / n (reference n = 100)              */
  int32_t output;          /* enum jsh_output                                       */
  int32_t precision;       /* enum jsh_precision                                    */
  int32_t schedule;        /* enum jsh_schedule                                     */
  double tau_max;          /* stop the tau pass at tau >= tau_max (reference 1e4)   */
  double tau_min;          /* run the I pass only if tau > tau_min (1e-10)          */
  double dt_max;           /* [cm] largest tau-pass step, 0 = no limit              */
  double tau_atol;         /* tau pass tolerances (reference 1e-7, 1e-14)           */
  double tau_rtol;
  double atol;             /* I / IQUV pass tolerances (reference 1e-9, 1e-9)        */
  double rtol;
  double tau_precision;    /* |tau - tau_max| target of the crossing bisection (1)   */
  int64_t max_steps;       /* accepted+rejected steps per segment and pass (0: 1<<22)*/
  int32_t block_size;      /* 0 = autotuned / default                               */
  int32_t refill_threshold;/* persistent schedule: refill when this many lanes idle  */
  int32_t ctas_per_sm;     /* persistent schedule: 0 = occupancy maximum             */
  int32_t flags;           /* JSH_FLAG_* (0 = defaults)                              */
} jsh_params;

/* Mixed precision: start the IQUV pass of an optically thick ray inside it
 * instead of at tau_max.  With tau_thick = 16 / (1 - p) (p = k_Q / k_I +
 * 0.05, at most 0.95; p = 0 for I-only output) the Stokes vector entering at
 * tau_thick reaches the observer attenuated by at least exp(-16) ~ 1.1e-7.
 * I-only output starts there from the zero state.  Full Stokes output starts
 * a ray deeper than tau_thick at optical depth 30 from the local equilibrium
 * x = K^-1 eps of the transfer matrix (the true state there differs from it
 * only through the source function's gradients; measured worst 2.2e-6 of I
 * against the integration from tau_max).  Thick rays need a small fraction
 * of the stiff IQUV steps.  This flag turns it off (integrate from tau_max
 * like src/Observation.cpp:242-274).  The FP64 path always integrates from
 * tau_max. */
#define JSH_FLAG_IQUV_FROM_TAU_MAX 0x1
/* Cost map: the l plane receives each item's number of right-hand-side
 * evaluations instead of the path length (schedule and cost studies). */
#define JSH_FLAG_COST_MAP 0x2
/* Mixed persistent schedule: launch the register-capped build of the
 * transfer kernel (at most 128 threads per CTA; more resident warps per SM).
 * Results are bitwise those of the default build; jsh_autotune chooses
 * between the two for requests that leave the launch knobs at 0. */
#define JSH_FLAG_COMPACT_REGS 0x4
/* Mixed persistent schedule: run each item's tau pass and I/IQUV pass in one
 * persistent kernel, whose warps mix lanes of both passes, instead of the
 * default split (a tau kernel over every item, then an IQUV kernel over the
 * items that need the second pass, ranked by the optical depth it crosses).
 * Results are bitwise the same; the flag exists for comparison. */
#define JSH_FLAG_SINGLE_KERNEL 0x8
/* Split form: launch the kernels built for every field law even when the
 * model is of the benchmark family (helical conical B and BK n in the plasma
 * frame, ConstFlat V), whose requests otherwise run kernels compiled with
 * that family's fused coefficient path alone (fewer registers, more
 * resident warps).  Results are bitwise the same; for comparison. */
#define JSH_FLAG_GENERAL_KERNELS 0x10
/* Mixed persistent schedule: record CUDA events on the launching stream
 * around the tau kernel, the IQUV ranking kernels and the IQUV kernel, read
 * back with jsh_last_kernel_ms (per-kernel device time for roofline
 * figures).  Results are unchanged. */
#define JSH_FLAG_KERNEL_TIMES 0x20
/* Split form, requests of at least 65536 work items: overlap the passes.
 * The rays estimated deepest (the optical depth of the ranking >= 8 at the
 * first frequency) run their tau pass first, then their IQUV pass, which
 * holds the render's longest items, at high priority beside the other rays'
 * tau and IQUV passes (a second stream of the context, joined before the
 * call's work ends on the caller's stream).  It pays when those items set
 * the render's length; jsh_autotune tries it and keeps it for the context
 * when faster (JSH_FLAG_SERIAL_PASSES then runs one serial chain).  With
 * overlapped passes the times of JSH_FLAG_KERNEL_TIMES are those of the
 * phases: both tau kernels, the other rays' IQUV ranking, and the rest.
 * Results are bitwise the same either way. */
#define JSH_FLAG_SERIAL_PASSES 0x40
#define JSH_FLAG_OVERLAP_PASSES 0x80
/* Mixed precision, full Stokes: the Faraday-thick mode of the I/IQUV pass.
 * Where Faraday rotation outruns absorption a hundredfold (|k_F| >= 100 k_I)
 * the pass follows (Q, U) at its quasi-static value S / (k_I - i k_F) plus a
 * decaying transient and steps on I and V alone, within the request's
 * rtol/atol relative to I; it returns to the full integration where the
 * adiabatic condition fails, near the jet axis and where k_F changes sign.
 * Faraday-thick jet cores take thousands of times fewer steps.  The request
 * runs kernels built with the mode (the default kernels leave its
 * bookkeeping out); images of jets without Faraday-thick rays are the same
 * to the last bit either way.  The FP64 path never uses it. */
#define JSH_FLAG_FARADAY_THICK 0x100

/* Fill *p with the reference's hard-coded values (src/pyjetshow.cpp:143-156,
 * src/Observation.cpp:156, :269): n = 100, tau_max = 1e4, tau_min = 1e-10,
 * dt_max = 0, tau tolerances (1e-7, 1e-14), I tolerances (1e-9, 1e-9),
 * tau_precision = 1, output I, FP64, static schedule. */
void jsh_params_default(jsh_params* p);

/* --------------------------------------------------------------- outputs */
typedef struct jsh_image {
  /* Each non-NULL plane holds n_nu * n_across * n_along values. */
  double* tau;
  double* l;      /* untruncated path length through the jet [cm] */
  double* I;
  double* Q;
  double* U;
  double* V;
  uint32_t* status;
} jsh_image;

typedef struct jsh_stats {
  uint64_t n_pixels;
  uint64_t n_hit_pixels;    /* pixels whose ray intersects the geometry  */
  uint64_t n_work_items;    /* hit pixels x frequencies                   */
  uint64_t rhs_evals;       /* right-hand-side evaluations on the device  */
  uint64_t steps_accepted;
  uint64_t steps_rejected;
  uint32_t status_or;       /* OR of all per-item status bits             */
  uint32_t kernels_launched;
  double device_ms;         /* CUDA-event time of the render kernels      */
  double total_ms;          /* host wall time of the call                 */
} jsh_stats;

/* ------------------------------------------------------------- context */
typedef struct jsh_ctx jsh_ctx;

int jsh_abi_version(void);
const char* jsh_last_error(void); /* thread-local message of the last failure */

/* Create a context on CUDA device `device`.  hbm_budget_bytes caps the device
 * memory the context may hold for requests (0 = 80% of free memory). */
int jsh_ctx_create(int device, uint64_t hbm_budget_bytes, jsh_ctx** out);
void jsh_ctx_destroy(jsh_ctx* ctx);

/* Observation::run + getImage for n_nu frequencies in one call, host buffers
 * in and out (host<->device copies included).  nu_hz are source-frame
 * frequencies (the reference multiplies by 1e9 (1+z) before the call). */
int jsh_observation_run(jsh_ctx* ctx, const jsh_model_desc* model,
                        const jsh_plane_desc* plane, const double* nu_hz,
                        int32_t n_nu, const jsh_params* params,
                        jsh_image* host_out, jsh_stats* stats);

/* Same, but the outputs are DEVICE pointers and the work is enqueued on
 * `cuda_stream` (a cudaStream_t, NULL = legacy default stream).  The call
 * returns after enqueueing; the caller synchronises the stream. */
int jsh_observation_run_device(jsh_ctx* ctx, const jsh_model_desc* model,
                               const jsh_plane_desc* plane, const double* nu_hz,
                               int32_t n_nu, const jsh_params* params,
                               void* cuda_stream, jsh_image* device_out);

/* Device counters of the last jsh_observation_run_device call on this
 * context (synchronises the context's work first). */
int jsh_last_stats(jsh_ctx* ctx, jsh_stats* stats);

/* Allocation-free form of jsh_observation_run_device, for callers that must
 * not allocate device memory: hosts whose framework owns the whole device
 * memory pool and forbids side allocations, and latency-bound loops that
 * cannot take the implicit device synchronisation of cudaMalloc/cudaFree.
 * No context: it renders on the current device, enqueued on `cuda_stream`,
 * into the caller's DEVICE output planes, and calls no cudaMalloc, cudaFree
 * or other allocating routine.  The host inputs travel as kernel parameters
 * (nothing reads the caller's host memory after the call returns).  Its
 * scratch is one 8 MiB file-scope device array that every GPU loading the
 * library holds until exit; it limits a call to JSH_NOALLOC_MAX_PIXELS
 * pixels, JSH_NOALLOC_MAX_ALONG columns, JSH_NOALLOC_MAX_NU frequencies and
 * analytic fields and geometries (no grids, no hulls), and rejects larger
 * requests with JSH_ERR_INVALID.  Calls share the array and it keeps the
 * last call's contents: each call clears what must start at zero, and calls
 * that overlap on the GPU race.  The first call on a device looks up the
 * array's address; make it before any stream capture.  No counterpart in
 * the reference, which renders on the CPU. */
#define JSH_NOALLOC_MAX_PIXELS 65536
#define JSH_NOALLOC_MAX_ALONG 4096
#define JSH_NOALLOC_MAX_NU 64
int jsh_observation_run_noalloc(const jsh_model_desc* model, const jsh_plane_desc* plane, const double* nu_hz,
                                int32_t n_nu, const jsh_params* params, void* cuda_stream,
                                jsh_image* device_out);

/* ------------------------------------------------------- visibilities */
/* The visibility step after the render (JetModelZoom.ft, jetmodel.py:114-132,
 * with FINUFFT_NUNU's type-3 transform, fourier.py:40-94): for every
 * frequency f and (u, v) point k,
 *   V = exp(-2 pi i (u dx + v dy)) sum_j F_j exp(-2 pi i (u' x_j + v' y_j)),
 *   (u', v') = (u cos rot + v sin rot, -u sin rot + v cos rot),
 * over the image's pixel centres x_j = -across_j rad_per_cm,
 * y_j = along_j rad_per_cm and flux densities F_j = I_j size_j^2 jy_per_cgs
 * (size_j the pixel side in cm).  get_i_image's Jy conversion
 * (src/pyjetshow.cpp:111-169) is jy_per_cgs = 1e23 (1+z)^-3
 * (mas_to_rad / (pc_in_mas pc))^2; rad_per_cm = 1 / D_A. */
typedef struct jsh_vis_desc {
  double rad_per_cm;  /* angle of 1 cm at the source [rad/cm] (> 0)            */
  double jy_per_cgs;  /* flux density per (I [cgs] x pixel area [cm^2])        */
  double dx, dy;      /* [rad] shift of the model on the sky                   */
  double rot;         /* [rad] rotation of the (u, v) plane                    */
} jsh_vis_desc;

/* Render (like jsh_observation_run, with the outputs kept on the device)
 * and transform the Stokes I image of every frequency: uv[n_nu][n_uv][2]
 * in wavelengths (host), vis_out[n_nu][n_uv][2] (re, im) in Jy (host).  The
 * sum is evaluated directly on the device (no gridding approximation;
 * ~1e-7 relative to an FP64 direct sum).  n_across <= 16384. */
int jsh_observation_visibilities(jsh_ctx* ctx, const jsh_model_desc* model,
                                 const jsh_plane_desc* plane, const double* nu_hz,
                                 int32_t n_nu, const jsh_params* params,
                                 const jsh_vis_desc* vis, const double* uv,
                                 int64_t n_uv, double* vis_out, jsh_stats* stats);

/* Stripe mode (Observation::run_stripe + getStripe, src/Observation.cpp:310-347,
 * src/Image.cpp:31-41): tau only, for the pixels of row n_across/2 from
 * column n_along/2 to the end, in FP64 on the device with the reference's
 * integrate_tau (src/Observation.cpp:55-123): n constant RK4 steps per
 * intersection, stopped at the first step whose tau >= tau_max.
 * tau_host[n_along - n_along/2] (host buffer); nu_hz source-frame. */
int jsh_observation_run_stripe(jsh_ctx* ctx, const jsh_model_desc* model,
                               const jsh_plane_desc* plane, double nu_hz, int32_t n,
                               double tau_max, double* tau_host);

/* Ray generation on the device (ImagePlane + Image + Ray ctors): origins
 * [n_across*n_along][3], the common unit direction [3], pixel sizes
 * [n_across*n_along] (cm), all host buffers (any may be NULL). */
int jsh_plane_rays(jsh_ctx* ctx, const jsh_plane_desc* plane, double* origins,
                   double* direction, double* pixel_sizes);

/* Geometry hit of every pixel's ray on the device.  n_seg[pix] in {0,1,2};
 * seg[pix][k] = {point_in xyz, point_out xyz} (k < 2), host buffers. */
int jsh_trace_plane(jsh_ctx* ctx, const jsh_model_desc* model,
                    const jsh_plane_desc* plane, int32_t* n_seg, double* seg,
                    uint32_t* status);

/* Geometry hit of arbitrary rays (origins[n][3], directions[n][3], the
 * directions are normalised like Ray::Ray).  Same outputs as above. */
int jsh_hit_rays(jsh_ctx* ctx, const jsh_model_desc* model, const double* origins,
                 const double* directions, int64_t n, int32_t* n_seg,
                 double* seg, uint32_t* status);

/* --------------------------------------------------------- cosmology */
typedef struct jsh_cosmology {
  double H0;       /* km/s/Mpc (reference default 69.32)          */
  double omega_M;  /* (0.2865)                                    */
  double omega_V;  /* (0.7134130719051658)                        */
  double gamma_nu; /* (8.69280948342326e-05)                      */
} jsh_cosmology;

/* Parsecs per milliarcsecond at redshift z (mas_to_pc, src/utils.cpp:205-208).
 * cosmo == NULL selects the reference defaults. */
double jsh_mas_to_pc(double z, const jsh_cosmology* cosmo);

/* --------------------------------------------------------- gridded fields */
/* Delaunay triangulation of n points (xy[n][2]) on the host.  tri_out must
 * hold 3*(2n) int32; *n_tri receives the triangle count. */
int jsh_grid_triangulate(const double* xy, int64_t n, int32_t* tri_out,
                         int64_t* n_tri);

/* Upload a triangulated (z, r) grid once: xy[n][2] in pc (z, r), values
 * [n][n_fields] FP32, tri[n_tri][3].  Returns a grid id for field
 * descriptors (JSH_*_SIMULATION). */
int jsh_grid_upload(jsh_ctx* ctx, const double* xy, int64_t n_points,
                    const float* values, int32_t n_fields, const int32_t* tri,
                    int64_t n_tri, int32_t* grid_id);

/* Interpolate field `field` of a grid at host points (z, r) in pc on the
 * device (SimulationInterpolater::interpolated_value).  out[n]. */
int jsh_grid_interpolate(jsh_ctx* ctx, int32_t grid_id, int32_t field,
                         const double* zr, int64_t n, double nan_value,
                         double* out);

/* --------------------------------------------------- simulation geometry */
/* The jet boundary of a gridded simulation (SimulationGeometry,
 * src/Geometry.cpp:92-132): the convex hull of the (z, r) points zr[n][2]
 * (pc) revolved about the z axis at n_circle azimuths phi_j = 2 pi j /
 * n_circle, the point (r sin phi_j, r cos phi_j, z) (the reference builds it
 * with n_circle = 36, src/main.cpp:880-897).  That hull is the set of points
 * whose n_circle-gon "radius" about the axis is at most R(z), R the upper
 * envelope of the convex hull of the (z, r) profile, so only the profile is
 * stored (host-built once, a few KB on the device).  A ray's segment is the
 * whole line's intersection with the hull (the reference intersects the
 * line, not the half-line), point_in at the smaller ray parameter.  Requires
 * r >= 0, n >= 2 and two distinct z values; 3 <= n_circle <= 4096.  Returns a
 * hull id for jsh_geometry_desc.hull_id (kind JSH_GEO_SIMULATION). */
#define JSH_MAX_HULLS 16
int jsh_hull_upload(jsh_ctx* ctx, const double* zr, int64_t n, int32_t n_circle,
                    int32_t* hull_id);
/* The profile jsh_hull_upload stores, computed on the host only (no device,
 * no context): the vertices (vz[i], vR[i]), i = 0..*m, of R(z); vz and vR
 * must hold n entries.  Same argument checks as jsh_hull_upload. */
int jsh_hull_profile(const double* zr, int64_t n, int32_t n_circle, double* vz,
                     double* vR, int32_t* m);

/* ---------------------------------------------------- random cells */
/* The cells of RandomCellsInSphere::create (src/Cells.cpp:35-47): n points
 * drawn as generate_random_points_sphere does (src/utils.cpp:267-312):
 *   r = r_min + (r_max - r_min) U1, phi = 2 pi U2,
 *   u = (1 - c)(2 U3 - 1) shifted by -c (u < 0) or +c, c = cos(theta_max)
 *   (c = 1 for theta_max <= 0: every point on the axis, as there),
 *   theta = acos(u), r = r^(1 / (3 - exponent)),
 *   point = (r sin theta cos phi, r sin theta sin phi, r cos theta) [cm],
 * and one random unit direction per cell (generate_random_directions,
 * src/utils.cpp:249-261).  The reference's Boost Mersenne Twister streams
 * are replaced by Philox4x32-10 keyed by `seed` (uniforms U = (x + 1/2)
 * 2^-32 of its 32-bit outputs).  Host only (no context, no device).  All n
 * points are kept (the reference copies only the first n/2 into its cell
 * matrix and leaves the rest uninitialised). */
int jsh_cells_generate(int64_t n, double r_min, double r_max, double theta_max, double exponent, uint64_t seed,
                       double* points, double* directions);
/* Upload a cell set (points[n][3] cm, unit directions[n][3]) once; returns
 * an id for jsh_random_desc.cells_id.  The device finds a point's cell
 * through a uniform bucket grid whose buckets list every point that can be
 * nearest inside them (exact: the nearest point, ties to the lowest index). */
#define JSH_MAX_CELLS 16
int jsh_cells_upload(jsh_ctx* ctx, const double* points, const double* directions, int64_t n, int32_t* cells_id);
/* Checks: the nearest cell of each of n host points (cm), found on the
 * device (out[n]); the random unit directions for n counters keys[n][3]
 * (k0, k1, k2) of `seed`, drawn on the device (out[n][3]). */
int jsh_cells_nearest(jsh_ctx* ctx, int32_t cells_id, const double* points, int64_t n, int32_t* out);
int jsh_random_directions(jsh_ctx* ctx, uint64_t seed, const uint32_t* keys, int64_t n, double* out);

/* --------------------------------------------------------- serving */
typedef struct jsh_server jsh_server;
typedef uint64_t jsh_request_id;

typedef struct jsh_server_config {
  int32_t max_inflight_batches; /* concurrent device batches (streams), >= 1 */
  int32_t max_batch_requests;   /* requests merged into one device batch      */
  int32_t precision;            /* enum jsh_precision for every request       */
  int32_t use_graphs;           /* capture each batch's launch sequence       */
  uint64_t hbm_budget_bytes;    /* device memory the queue may hold (0: ctx)  */
} jsh_server_config;

typedef struct jsh_request_stats {
  double queue_ms;    /* submit -> admitted                               */
  double service_ms;  /* admitted -> result on host                       */
  double latency_ms;  /* submit -> result on host                         */
  uint64_t n_work_items;
  uint32_t status_or;
  int32_t batch_size; /* requests in the device batch this one ran in     */
} jsh_request_stats;

int jsh_server_create(jsh_ctx* ctx, const jsh_server_config* cfg,
                      jsh_server** out);
void jsh_server_destroy(jsh_server* srv);
/* Enqueue a render; copies every descriptor and nu_hz.  Never blocks on the
 * device.  JSH_ERR_OOM if the request alone exceeds the HBM budget. */
int jsh_server_submit(jsh_server* srv, const jsh_model_desc* model,
                      const jsh_plane_desc* plane, const double* nu_hz,
                      int32_t n_nu, const jsh_params* params,
                      jsh_request_id* id);
/* 1 if finished, 0 if not yet, negative on error. */
int jsh_server_poll(jsh_server* srv, jsh_request_id id);
/* Wait up to timeout_ms (< 0: forever) and copy the result planes into
 * host_out (planes may be NULL); releases the request. */
int jsh_server_wait(jsh_server* srv, jsh_request_id id, int32_t timeout_ms,
                    jsh_image* host_out, jsh_request_stats* stats);
/* Cancel a request that has not been admitted yet. */
int jsh_server_cancel(jsh_server* srv, jsh_request_id id);

/* --------------------------------------------------------- autotuning */
typedef struct jsh_tuning {
  int32_t block_size;
  int32_t ctas_per_sm;
  int32_t refill_threshold;
  int32_t compact;      /* 1: the register-capped build (JSH_FLAG_COMPACT_REGS) */
  int32_t overlap;      /* 1: overlapped passes (JSH_FLAG_OVERLAP_PASSES) */
  double ms;            /* best measured time */
} jsh_tuning;

/* Time the persistent schedule over a grid of kernel builds (default and
 * register-capped), block sizes, CTAs per SM, refill thresholds and serial
 * or overlapped passes on this request and store the fastest in the
 * context; later requests with block_size == 0 use it (the overlap choice
 * holds unless a request's flags force one). */
int jsh_autotune(jsh_ctx* ctx, const jsh_model_desc* model,
                 const jsh_plane_desc* plane, const double* nu_hz,
                 int32_t n_nu, const jsh_params* params, jsh_tuning* best);

/* --------------------------------------------------------- diagnostics */
/* Measured issue rates of the context's device, for roofline fractions of
 * the compute-bound transfer kernels: FP32 FMA throughput (TFLOP/s, two
 * flops per FMA), MUFU ex2 throughput (T ops/s) and FP64 FMA throughput
 * (TFLOP/s), each from a dependent-chain microbenchmark over every SM.
 * No reference counterpart (the reference has no device code). */
int jsh_device_peaks(jsh_ctx* ctx, double* fp32_tflops, double* mufu_tops, double* fp64_tflops);

/* Device times [ms] of the last request enqueued on the context with
 * JSH_FLAG_KERNEL_TIMES on the mixed persistent schedule: the tau kernel,
 * the IQUV ranking kernels and the IQUV kernel (the single-kernel form
 * reports its one kernel as iquv_ms and 0 for the others; overlapped passes
 * report phases, see JSH_FLAG_SERIAL_PASSES).  Waits for the
 * request's kernels.  JSH_ERR_NOT_FOUND when the last request did not ask
 * for them.  No reference counterpart. */
int jsh_last_kernel_ms(jsh_ctx* ctx, double* tau_ms, double* iquv_rank_ms, double* iquv_ms);

/* Host-to-device bytes that one jsh_observation_run or
 * jsh_observation_run_device call copies: the compiled request record, the
 * n_nu frequencies and, for JSH_PREC_MIXED, their FP32 coefficient
 * constants.  The descriptors themselves are read on the host.  No device
 * work; no reference counterpart. */
uint64_t jsh_request_h2d_bytes(int32_t n_nu, int32_t precision);

/* The panel rule of the mixed-precision tau pass for the smooth benchmark
 * family (helical conical B and BK n in the plasma frame, flat flow): the
 * 7/15-point Gauss-Kronrod rule on [-1, 1], 15 nodes ascending (x), Kronrod
 * weights (wk) and Gauss weights (wg, zero at the Kronrod-only nodes), in
 * FP64; the device holds them in FP32 on [0, 1].  For tests of the rule;
 * no device work, no reference counterpart (the reference integrates tau
 * with Dormand-Prince steps, src/Observation.cpp:150-211). */
void jsh_tau_panel_rule(double* x, double* wk, double* wg);

#ifdef __cplusplus
}
#endif

#endif /* JETSHOW_CAPI_H */
