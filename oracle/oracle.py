"""TEST INFRASTRUCTURE: ctypes loader of the CPU oracle (``oracle/jsh_oracle.c``).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker.  The oracle is an
FP64 restatement of the reference path; parity is pinned by the reference's
Cone::hit golden vectors and by analytic known answers (see ``tests/``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from jetshow_gb300 import _capi as A

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libjsh_oracle.so")


class Counters(C.Structure):
    _fields_ = [("rhs_evals", C.c_uint64), ("steps_accepted", C.c_uint64),
                ("steps_rejected", C.c_uint64)]


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off, OpenMP)."""
    r = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        # retry without OpenMP (a toolchain without libgomp)
        r = subprocess.run(["make", "-C", HERE, "OMPFLAGS="], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        P, D = C.POINTER, C.POINTER(C.c_double)
        L.jo_plane_rays.argtypes = [P(A.PlaneDesc), D, D, D]
        L.jo_hit_rays.argtypes = [P(A.ModelDesc), D, D, C.c_int64, P(C.c_int32), D, P(C.c_uint32)]
        L.jo_set_item_evals.argtypes = [P(C.c_uint64)]
        L.jo_set_item_evals.restype = None
        L.jo_render.argtypes = [P(A.ModelDesc), P(A.PlaneDesc), D, C.c_int32, P(A.Params),
                                P(C.c_int64), C.c_int64, C.c_int32, P(A.Image), P(Counters)]
        L.jo_coefficients.argtypes = [P(A.ModelDesc), D, D, C.c_double, D]
        L.jo_fields.argtypes = [P(A.ModelDesc), D, D]
        L.jo_steps_schedule.argtypes = [C.c_double, C.c_int, C.c_int]
        L.jo_steps_schedule.restype = C.c_int
        L.jo_test_linear_dense.argtypes = [C.c_double] * 6 + [P(C.c_int64)]
        L.jo_test_linear_dense.restype = C.c_double
        L.jo_test_linear_controlled.argtypes = [C.c_double] * 6 + [P(C.c_int64)]
        L.jo_test_linear_controlled.restype = C.c_double
        L.jo_test_dense_error.argtypes = [C.c_double, C.c_double]
        L.jo_test_dense_error.restype = C.c_double
        L.jo_mas_to_pc.argtypes = [C.c_double, P(A.Cosmology)]
        L.jo_mas_to_pc.restype = C.c_double
        L.jo_grid_register.argtypes = [C.c_int32, D, C.c_int64, P(C.c_float), C.c_int32,
                                       P(C.c_int32), C.c_int64]
        L.jo_grid_value.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double]
        L.jo_grid_value.restype = C.c_double
        L.jo_stripe.argtypes = [P(A.ModelDesc), P(A.PlaneDesc), C.c_double, C.c_int32, C.c_double, D]
        L.jo_hull_register.argtypes = [C.c_int32, D, C.c_int64, C.c_int32]
        L.jo_hull_profile.argtypes = [C.c_int32, D, D, P(C.c_int32)]
        L.jo_openmp_threads.restype = C.c_int
        L.jo_philox4x32.argtypes = [P(C.c_uint32), C.c_uint64, P(C.c_uint32)]
        L.jo_random_direction.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, D]
        L.jo_random_direction.restype = None
        L.jo_cells_generate.argtypes = [C.c_int64, C.c_double, C.c_double, C.c_double, C.c_double, C.c_uint64, D, D]
        L.jo_cells_register.argtypes = [C.c_int32, D, D, C.c_int64]
        L.jo_cells_nearest.argtypes = [C.c_int32, D]
        L.jo_cells_nearest.restype = C.c_int64
        _lib = L
    return _lib


def _chk(st):
    if st != 0:
        raise RuntimeError(f"oracle call failed with status {st}")


def plane_rays(plane: A.PlaneDesc):
    n = int(plane.n_across * plane.n_along)
    o = np.zeros((n, 3)); d = np.zeros(3); s = np.zeros(n)
    _chk(lib().jo_plane_rays(C.byref(plane), A.dptr(o), A.dptr(d), A.dptr(s)))
    return o, d, s


def hit_rays(model: A.ModelDesc, origins, directions):
    origins = np.ascontiguousarray(origins, dtype=np.float64)
    directions = np.ascontiguousarray(directions, dtype=np.float64)
    n = origins.shape[0]
    nseg = np.zeros(n, np.int32); seg = np.zeros((n, 2, 2, 3)); st = np.zeros(n, np.uint32)
    _chk(lib().jo_hit_rays(C.byref(model), A.dptr(origins), A.dptr(directions), n,
                           nseg.ctypes.data_as(C.POINTER(C.c_int32)), A.dptr(seg),
                           st.ctypes.data_as(C.POINTER(C.c_uint32))))
    return nseg, seg, st


def render(model: A.ModelDesc, plane: A.PlaneDesc, nu, params: A.Params, pix=None, threads=0, item_evals=False):
    """Render (all pixels or the flat pixel indices ``pix``); returns a dict of
    [n_nu, n_sel] arrays plus counters (and the per-item RHS evaluation
    counts as ``evals`` when ``item_evals``)."""
    nu = np.ascontiguousarray(np.atleast_1d(nu), dtype=np.float64)
    npix = int(plane.n_across * plane.n_along)
    if pix is None:
        nsel = npix
        pix_p = None
    else:
        pix = np.ascontiguousarray(pix, dtype=np.int64)
        nsel = pix.size
        pix_p = pix.ctypes.data_as(C.POINTER(C.c_int64))
    out = {k: np.zeros((nu.size, nsel)) for k in ("tau", "l", "I", "Q", "U", "V")}
    out["status"] = np.zeros((nu.size, nsel), np.uint32)
    img = A.Image(*(A.dptr(out[k]) for k in ("tau", "l", "I", "Q", "U", "V")),
                  out["status"].ctypes.data_as(C.POINTER(C.c_uint32)))
    cnt = Counters()
    if item_evals:
        out["evals"] = np.zeros((nu.size, nsel), np.uint64)
        lib().jo_set_item_evals(out["evals"].ctypes.data_as(C.POINTER(C.c_uint64)))
    try:
        _chk(lib().jo_render(C.byref(model), C.byref(plane), A.dptr(nu), nu.size, C.byref(params),
                             pix_p, nsel, threads, C.byref(img), C.byref(cnt)))
    finally:
        if item_evals:
            lib().jo_set_item_evals(None)
    out["rhs_evals"] = cnt.rhs_evals
    out["steps_accepted"] = cnt.steps_accepted
    out["steps_rejected"] = cnt.steps_rejected
    return out


def coefficients(model, point, n_los, nu):
    out = np.zeros(11)
    p = np.ascontiguousarray(point, dtype=np.float64)
    n = np.ascontiguousarray(n_los, dtype=np.float64)
    _chk(lib().jo_coefficients(C.byref(model), A.dptr(p), A.dptr(n), nu, A.dptr(out)))
    return out


def fields(model, point):
    """B (3; a scalar law's |B| first), n and v (3) [cm/s] of the model's
    laws at a lab-frame point [cm]."""
    out = np.zeros(7)
    p = np.ascontiguousarray(point, dtype=np.float64)
    _chk(lib().jo_fields(C.byref(model), A.dptr(p), A.dptr(out)))
    return out


def mas_to_pc(z, cosmo=None):
    return lib().jo_mas_to_pc(z, C.byref(cosmo) if cosmo is not None else None)


def grid_register(grid_id, xy, values, tri):
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    values = np.ascontiguousarray(values, dtype=np.float32)
    if values.ndim == 1:
        values = values[:, None]
    tri = np.ascontiguousarray(tri, dtype=np.int32)
    _chk(lib().jo_grid_register(grid_id, A.dptr(xy), xy.shape[0],
                                values.ctypes.data_as(C.POINTER(C.c_float)), values.shape[1],
                                tri.ctypes.data_as(C.POINTER(C.c_int32)), tri.shape[0]))


def grid_value(grid_id, field, z_pc, r_pc, nan_value=0.0):
    return lib().jo_grid_value(grid_id, field, z_pc, r_pc, nan_value)


def stripe(model: A.ModelDesc, plane: A.PlaneDesc, nu: float, n: int = 100, tau_max: float = 1e4):
    """tau along half of the central row (Observation::run_stripe)."""
    out = np.zeros(int(plane.n_along - plane.n_along // 2))
    _chk(lib().jo_stripe(C.byref(model), C.byref(plane), float(nu), int(n), float(tau_max), A.dptr(out)))
    return out


def hull_register(hull_id, zr, n_circle=36):
    zr = np.ascontiguousarray(zr, dtype=np.float64).reshape(-1, 2)
    _chk(lib().jo_hull_register(hull_id, A.dptr(zr), zr.shape[0], int(n_circle)))


def hull_profile(hull_id):
    """(z, R) vertices of a registered hull's profile."""
    m = C.c_int32()
    _chk(lib().jo_hull_profile(hull_id, None, None, C.byref(m)))
    vz = np.zeros(m.value + 1); vr = np.zeros(m.value + 1)
    _chk(lib().jo_hull_profile(hull_id, A.dptr(vz), A.dptr(vr), C.byref(m)))
    return vz, vr


def threads():
    return lib().jo_openmp_threads()


def philox4x32(ctr, key):
    c = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    out = (C.c_uint32 * 4)()
    _chk(lib().jo_philox4x32(c, int(key), out))
    return [int(x) for x in out]


def random_directions(seed, keys):
    """Unit directions [n, 3] of the counters keys [n, 3] (k0, k1, k2)."""
    keys = np.asarray(keys, dtype=np.uint32).reshape(-1, 3)
    out = np.zeros((keys.shape[0], 3))
    d = np.zeros(3)
    for i, (a, b, c) in enumerate(keys):
        lib().jo_random_direction(int(seed), int(a), int(b), int(c), A.dptr(d))
        out[i] = d
    return out


def cells_generate(n, r_min, r_max, theta_max, exponent, seed):
    p = np.zeros((n, 3)); d = np.zeros((n, 3))
    _chk(lib().jo_cells_generate(n, r_min, r_max, theta_max, exponent, int(seed), A.dptr(p), A.dptr(d)))
    return p, d


def cells_register(cells_id, points, dirs):
    points = np.ascontiguousarray(points, dtype=np.float64); dirs = np.ascontiguousarray(dirs, dtype=np.float64)
    _chk(lib().jo_cells_register(cells_id, A.dptr(points), A.dptr(dirs), points.shape[0]))


def cells_nearest(cells_id, q):
    q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
    return np.array([lib().jo_cells_nearest(cells_id, A.dptr(np.ascontiguousarray(x))) for x in q], dtype=np.int64)
