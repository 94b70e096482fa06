"""ctypes mirror of ``include/jetshow_capi.h``.

The structures and constants here are byte-for-byte the C-ABI declared in
``include/jetshow_capi.h``; ``load_library`` binds the in-tree
``libjetshow_gb300.so`` built by ``jetshow_gb300.build``.  There is no CPU
fallback: if the CUDA library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

# ----------------------------------------------------------------- status
JSH_OK = 0
JSH_ERR_INVALID = -1
JSH_ERR_CUDA = -2
JSH_ERR_OOM = -3
JSH_ERR_TIMEOUT = -4
JSH_ERR_NOT_FOUND = -5
JSH_ERR_NO_DEVICE = -6
JSH_ERR_CANCELLED = -7

ST_HIT = 0x1
ST_TAU_CROSSED = 0x2
ST_STEP_LIMIT = 0x4
ST_FAIL_LIMIT = 0x8
ST_BISECT_LIMIT = 0x10
ST_NAN = 0x20
ST_UB_GEOMETRY = 0x40
ST_DT_UNDERFLOW = 0x80
ST_IQUV = 0x100
FLAG_IQUV_FROM_TAU_MAX = 0x1
FLAG_COST_MAP = 0x2
FLAG_COMPACT_REGS = 0x4
FLAG_SINGLE_KERNEL = 0x8
FLAG_GENERAL_KERNELS = 0x10
FLAG_KERNEL_TIMES = 0x20
FLAG_SERIAL_PASSES = 0x40
FLAG_OVERLAP_PASSES = 0x80
FLAG_FARADAY_THICK = 0x100
ST_ERRORS = ST_STEP_LIMIT | ST_FAIL_LIMIT | ST_BISECT_LIMIT | ST_NAN | ST_DT_UNDERFLOW

GEO_CONE, GEO_CYLINDER, GEO_PARABALOID, GEO_PARABALOID_CONE, GEO_SIMULATION = 1, 2, 3, 4, 5

B_RANDOM_SCALAR = 1
B_RANDOM_SCALAR_Z = 2
B_COMPOSITE_RANDOM_SCALAR_Z = 3
B_CONST_CYLINDER = 10
B_CONST_CYLINDER_Z = 11
B_RADIAL_CONICAL = 12
B_TOROIDAL = 13
B_HELICAL_CYLINDER = 14
B_SPIRAL_CONICAL = 15
B_FORCE_FREE_CYLINDRICAL = 16
B_HELICAL_CONICAL = 17
B_SIMULATION = 20

N_CONST = 1
N_BK = 2
N_BKZ = 3
N_COMPOSITE_BK = 4
N_SIMULATION = 20

V_CONST_FLAT = 1
V_SHEARED_FLAT = 2
V_SHEATH_FLAT = 3
V_CONST_CENTRAL = 4
V_SHEARED_CENTRAL = 5
V_SHEATH_CENTRAL = 6
V_CONST_PARABOLIC = 7
V_ACC_PARABOLIC = 8
V_SHEARED_ACC_PARABOLIC = 9
V_ACC_PARABOLIC_CONST_CONE = 10
V_SHEARED_ACC_PARABOLIC_CONST_CONE = 11
V_SIMULATION = 20

OUT_I, OUT_FULL = 1, 2
PREC_FP64, PREC_MIXED = 1, 2
SCHED_STATIC, SCHED_PERSISTENT = 1, 2

SCALAR_B_KINDS = (B_RANDOM_SCALAR, B_RANDOM_SCALAR_Z, B_COMPOSITE_RANDOM_SCALAR_Z)


class GeometryDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("hull_id", C.c_int32),
        ("origin", C.c_double * 3),
        ("direction", C.c_double * 3),
        ("angle", C.c_double),
        ("big_scale", C.c_double),
        ("r", C.c_double),
        ("r0", C.c_double),
        ("z0", C.c_double),
    ]


class FieldDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("in_plasma_frame", C.c_int32),
        ("p", C.c_double * 8),
    ]


RND_NONE, RND_CELLS, RND_POINTS = 0, 1, 2


class RandomDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("cells_id", C.c_int32),
        ("fraction", C.c_double),
        ("seed", C.c_uint64),
    ]


class ModelDesc(C.Structure):
    _fields_ = [
        ("geometry", GeometryDesc),
        ("bfield", FieldDesc),
        ("nfield", FieldDesc),
        ("vfield", FieldDesc),
        ("s", C.c_double),
        ("gamma_min", C.c_double),
        ("thermal_fraction", C.c_double),
        ("random", RandomDesc),
    ]


class PlaneDesc(C.Structure):
    _fields_ = [
        ("n_across", C.c_uint64),
        ("n_along", C.c_uint64),
        ("lg_pixel_size_start_cm", C.c_double),
        ("lg_pixel_size_stop_cm", C.c_double),
        ("los_angle", C.c_double),
    ]


class Params(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("output", C.c_int32),
        ("precision", C.c_int32),
        ("schedule", C.c_int32),
        ("tau_max", C.c_double),
        ("tau_min", C.c_double),
        ("dt_max", C.c_double),
        ("tau_atol", C.c_double),
        ("tau_rtol", C.c_double),
        ("atol", C.c_double),
        ("rtol", C.c_double),
        ("tau_precision", C.c_double),
        ("max_steps", C.c_int64),
        ("block_size", C.c_int32),
        ("refill_threshold", C.c_int32),
        ("ctas_per_sm", C.c_int32),
        ("flags", C.c_int32),
    ]


class Image(C.Structure):
    _fields_ = [
        ("tau", C.POINTER(C.c_double)),
        ("l", C.POINTER(C.c_double)),
        ("I", C.POINTER(C.c_double)),
        ("Q", C.POINTER(C.c_double)),
        ("U", C.POINTER(C.c_double)),
        ("V", C.POINTER(C.c_double)),
        ("status", C.POINTER(C.c_uint32)),
    ]


class DeviceImage(C.Structure):
    """Same layout as ``Image`` with raw device addresses."""

    _fields_ = [
        ("tau", C.c_void_p),
        ("l", C.c_void_p),
        ("I", C.c_void_p),
        ("Q", C.c_void_p),
        ("U", C.c_void_p),
        ("V", C.c_void_p),
        ("status", C.c_void_p),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("n_pixels", C.c_uint64),
        ("n_hit_pixels", C.c_uint64),
        ("n_work_items", C.c_uint64),
        ("rhs_evals", C.c_uint64),
        ("steps_accepted", C.c_uint64),
        ("steps_rejected", C.c_uint64),
        ("status_or", C.c_uint32),
        ("kernels_launched", C.c_uint32),
        ("device_ms", C.c_double),
        ("total_ms", C.c_double),
    ]


class Cosmology(C.Structure):
    _fields_ = [
        ("H0", C.c_double),
        ("omega_M", C.c_double),
        ("omega_V", C.c_double),
        ("gamma_nu", C.c_double),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("max_inflight_batches", C.c_int32),
        ("max_batch_requests", C.c_int32),
        ("precision", C.c_int32),
        ("use_graphs", C.c_int32),
        ("hbm_budget_bytes", C.c_uint64),
    ]


class RequestStats(C.Structure):
    _fields_ = [
        ("queue_ms", C.c_double),
        ("service_ms", C.c_double),
        ("latency_ms", C.c_double),
        ("n_work_items", C.c_uint64),
        ("status_or", C.c_uint32),
        ("batch_size", C.c_int32),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("block_size", C.c_int32),
        ("ctas_per_sm", C.c_int32),
        ("refill_threshold", C.c_int32),
        ("compact", C.c_int32),
        ("overlap", C.c_int32),
        ("ms", C.c_double),
    ]


class VisDesc(C.Structure):
    _fields_ = [
        ("rad_per_cm", C.c_double),
        ("jy_per_cgs", C.c_double),
        ("dx", C.c_double),
        ("dy", C.c_double),
        ("rot", C.c_double),
    ]


_P = C.POINTER
_D = _P(C.c_double)

# (name, restype, argtypes) of every exported entry point of include/jetshow_capi.h
SIGNATURES = [
    ("jsh_abi_version", C.c_int, []),
    ("jsh_last_error", C.c_char_p, []),
    ("jsh_params_default", None, [_P(Params)]),
    ("jsh_ctx_create", C.c_int, [C.c_int, C.c_uint64, _P(C.c_void_p)]),
    ("jsh_ctx_destroy", None, [C.c_void_p]),
    ("jsh_observation_run", C.c_int,
     [C.c_void_p, _P(ModelDesc), _P(PlaneDesc), _D, C.c_int32, _P(Params), _P(Image), _P(Stats)]),
    ("jsh_observation_run_device", C.c_int,
     [C.c_void_p, _P(ModelDesc), _P(PlaneDesc), _D, C.c_int32, _P(Params), C.c_void_p, _P(DeviceImage)]),
    ("jsh_last_stats", C.c_int, [C.c_void_p, _P(Stats)]),
    ("jsh_observation_run_noalloc", C.c_int,
     [_P(ModelDesc), _P(PlaneDesc), _D, C.c_int32, _P(Params), C.c_void_p, _P(DeviceImage)]),
    ("jsh_observation_visibilities", C.c_int,
     [C.c_void_p, _P(ModelDesc), _P(PlaneDesc), _D, C.c_int32, _P(Params), _P(VisDesc), _D, C.c_int64, _D,
      _P(Stats)]),
    ("jsh_observation_run_stripe", C.c_int,
     [C.c_void_p, _P(ModelDesc), _P(PlaneDesc), C.c_double, C.c_int32, C.c_double, _D]),
    ("jsh_plane_rays", C.c_int, [C.c_void_p, _P(PlaneDesc), _D, _D, _D]),
    ("jsh_trace_plane", C.c_int,
     [C.c_void_p, _P(ModelDesc), _P(PlaneDesc), _P(C.c_int32), _D, _P(C.c_uint32)]),
    ("jsh_hit_rays", C.c_int,
     [C.c_void_p, _P(ModelDesc), _D, _D, C.c_int64, _P(C.c_int32), _D, _P(C.c_uint32)]),
    ("jsh_mas_to_pc", C.c_double, [C.c_double, _P(Cosmology)]),
    ("jsh_grid_triangulate", C.c_int, [_D, C.c_int64, _P(C.c_int32), _P(C.c_int64)]),
    ("jsh_grid_upload", C.c_int,
     [C.c_void_p, _D, C.c_int64, _P(C.c_float), C.c_int32, _P(C.c_int32), C.c_int64, _P(C.c_int32)]),
    ("jsh_grid_interpolate", C.c_int,
     [C.c_void_p, C.c_int32, C.c_int32, _D, C.c_int64, C.c_double, _D]),
    ("jsh_hull_upload", C.c_int, [C.c_void_p, _D, C.c_int64, C.c_int32, _P(C.c_int32)]),
    ("jsh_hull_profile", C.c_int, [_D, C.c_int64, C.c_int32, _D, _D, _P(C.c_int32)]),
    ("jsh_cells_generate", C.c_int,
     [C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double, C.c_uint64, _D, _D]),
    ("jsh_cells_upload", C.c_int, [C.c_void_p, _D, _D, C.c_int64, _P(C.c_int32)]),
    ("jsh_cells_nearest", C.c_int, [C.c_void_p, C.c_int32, _D, C.c_int64, _P(C.c_int32)]),
    ("jsh_random_directions", C.c_int, [C.c_void_p, C.c_uint64, _P(C.c_uint32), C.c_int64, _D]),
    ("jsh_server_create", C.c_int, [C.c_void_p, _P(ServerConfig), _P(C.c_void_p)]),
    ("jsh_server_destroy", None, [C.c_void_p]),
    ("jsh_server_submit", C.c_int,
     [C.c_void_p, _P(ModelDesc), _P(PlaneDesc), _D, C.c_int32, _P(Params), _P(C.c_uint64)]),
    ("jsh_server_poll", C.c_int, [C.c_void_p, C.c_uint64]),
    ("jsh_server_wait", C.c_int,
     [C.c_void_p, C.c_uint64, C.c_int32, _P(Image), _P(RequestStats)]),
    ("jsh_server_cancel", C.c_int, [C.c_void_p, C.c_uint64]),
    ("jsh_device_peaks", C.c_int, [C.c_void_p, _D, _D, _D]),
    ("jsh_request_h2d_bytes", C.c_uint64, [C.c_int32, C.c_int32]),
    ("jsh_last_kernel_ms", C.c_int, [C.c_void_p, _D, _D, _D]),
    ("jsh_tau_panel_rule", None, [_D, _D, _D]),
    ("jsh_autotune", C.c_int,
     [C.c_void_p, _P(ModelDesc), _P(PlaneDesc), _D, C.c_int32, _P(Params), _P(Tuning)]),
]

PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PACKAGE_DIR, "_build", "libjetshow_gb300.so")

_lib = None


def load_library(path: str | None = None):
    """Load and bind the CUDA library.  Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"jetshow_gb300 CUDA library not built ({p}); run jetshow_gb300.build.build() first")
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def dptr(a):
    """ctypes double* of a contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_D)
