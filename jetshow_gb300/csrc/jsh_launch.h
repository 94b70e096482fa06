// jsh_launch.h -- host-callable launchers of the device kernels.  A batch is
// an array of JshRequest in device memory; every launcher enqueues on
// `stream` and returns the cudaError_t of the launch.
#pragma once

#include <cuda_runtime.h>

#include "jsh_request.h"

#define JSH_MAX_BATCH 64
// Deep-prefix bucket of overlapped passes (estimated optical depth of a ray
// at the request's first frequency >= 8), and the smallest request (work
// items) that overlaps them.
#define JSH_OVERLAP_KEY 43
#define JSH_OVERLAP_MIN_ITEMS 65536

struct JshLaunchShape {
  int block_size;        // threads per CTA of the transfer kernel
  int ctas_per_sm;       // persistent schedule: CTAs per SM (0: occupancy max)
  int refill_threshold;  // persistent schedule: refill when >= this many lanes idle
  int compact;           // mixed persistent schedule: the 168-register build (<= 128 threads)
  int single;            // mixed persistent schedule: tau and IQUV passes in one kernel (else split)
  int fused;             // split form: every request of the batch is of the fused benchmark
                         // family (mix.helical_log): launch the kernels built for it alone
  // mixed persistent schedule, optional: four events recorded on the stream
  // before the tau kernel, after it, after the IQUV ranking and after the
  // IQUV kernel (the single-kernel form records only the last two;
  // with overlapped passes: before the deep prefix's tau kernel, after the
  // other rays' tau kernel and IQUV ranking, and after both IQUV kernels)
  cudaEvent_t* marks;
  // split form, optional: overlapped passes.  Rays whose rank bucket is at
  // least overlap_key (estimated optical depth >= 2^(overlap_key - 40)) form
  // the deep prefix: its tau pass runs first and its IQUV pass, which holds
  // the render's longest items, runs on `stream` at high priority while the
  // other rays' tau and IQUV passes run on `side` (fork[0] / fork[1]: events
  // of the fork and the join).  0 or no side stream: one serial chain.
  int overlap_key;
  cudaStream_t side;
  cudaEvent_t* fork;
  // mixed precision, full Stokes: run the kernels built with the
  // Faraday-thick mode (JSH_FLAG_FARADAY_THICK)
  int faraday_thick;
};

// Ray generation: along sizes and centres (sequential recurrence of
// pyLogspace / partial_sum), then the across-centre table.  max_along is
// the largest n_along of the batch.
cudaError_t jsh_launch_plane(const JshRequest* d_reqs, int n_req, uint64_t max_along, cudaStream_t stream);

// Hit every pixel's ray against the request's geometry, append the hit rays
// to req.hits (count in *req.n_hit, zeroed beforehand), write the outputs of
// missing pixels (zeros and geometry status) for every frequency.
cudaError_t jsh_launch_hit(const JshRequest* d_reqs, int n_req, uint64_t max_pix, cudaStream_t stream);

// Transfer every (hit ray, frequency) of the batch.  `queue` is a zeroed
// device counter used by the persistent schedule; max_items bounds the
// total work items (sum of npix * n_nu) for the static grid, max_hits the
// hit rays of one request.
cudaError_t jsh_launch_transfer(const JshRequest* d_reqs, int n_req, int precision, int schedule, bool full,
                                uint64_t max_items, uint64_t max_hits, const JshLaunchShape& shape,
                                unsigned int* queue, int num_sms, cudaStream_t stream);

// Hit arbitrary rays (origins/directions device arrays, directions already
// normalised on the device by this kernel as Ray::Ray does).
cudaError_t jsh_launch_hit_rays(const JshModel& model, const double* d_orig, const double* d_dir, int64_t n,
                                int32_t* d_nseg, double* d_seg, uint32_t* d_status, cudaStream_t stream);

// Plane rays (origins, sizes) of one compiled plane whose along/across tables
// are filled.
cudaError_t jsh_launch_plane_rays(const JshPlane& plane, double* d_orig, double* d_sizes, cudaStream_t stream);

// Gridded field interpolation at (z, r) points.
cudaError_t jsh_launch_grid_interp(const JshGrid& grid, int field, const double* d_zr, int64_t n,
                                   double nan_value, double* d_out, cudaStream_t stream);

// Largest resident CTAs per SM of the persistent transfer kernel whose launch
// shape the knobs set (mixed: the IQUV kernel of the split form, or the
// single-kernel form; compact: its register-capped build; 0 if it cannot run
// block_size threads).
int jsh_persistent_occupancy(int precision, bool full, int block_size, bool compact = false, bool single = false);

// Nearest cell of n points (cm) of an uploaded cell set (checks), and the
// random unit directions of n counters (k0, k1, k2) of `seed`.
cudaError_t jsh_launch_cells_nearest(const JshCells& cells, const double* d_pts, int64_t n, int32_t* d_out,
                                     cudaStream_t stream);
cudaError_t jsh_launch_random_directions(uint64_t seed, const uint32_t* d_keys, int64_t n, double* d_out,
                                         cudaStream_t stream);
