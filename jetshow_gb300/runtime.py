"""Process-level handle on the C-ABI context (``jsh_ctx``) and the calls the
Python host side makes through it.  Results come back as numpy arrays
shaped [n_nu, n_across, n_along]."""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _capi as A

PLANES = ("tau", "l", "I", "Q", "U", "V")


class JetshowError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"jetshow_gb300 error {status}: {msg}")
        self.status = status


def check(lib, st):
    if st != 0:
        raise JetshowError(st, (lib.jsh_last_error() or b"").decode(errors="replace"))
    return st


class Context:
    """Owns one ``jsh_ctx`` on a CUDA device."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.lib = A.load_library()
        h = C.c_void_p()
        check(self.lib, self.lib.jsh_ctx_create(device, hbm_budget_bytes, C.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self.lib.jsh_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------- render
    def render(self, model: A.ModelDesc, plane: A.PlaneDesc, nu, params: A.Params, want=PLANES):
        nu = np.ascontiguousarray(np.atleast_1d(nu), dtype=np.float64)
        na, nl = int(plane.n_across), int(plane.n_along)
        out = {k: np.zeros((nu.size, na, nl)) for k in want}
        out["status"] = np.zeros((nu.size, na, nl), np.uint32)
        img = A.Image(*(A.dptr(out[k]) if k in out else None for k in PLANES),
                      out["status"].ctypes.data_as(C.POINTER(C.c_uint32)))
        st = A.Stats()
        check(self.lib, self.lib.jsh_observation_run(self.handle, C.byref(model), C.byref(plane),
                                                     A.dptr(nu), nu.size, C.byref(params), C.byref(img),
                                                     C.byref(st)))
        return out, stats_dict(st)

    def render_device(self, model, plane, nu, params, stream_ptr, dev_planes: dict):
        """Enqueue a render on a CUDA stream with device output pointers
        (``dev_planes`` maps plane names to raw device addresses)."""
        nu = np.ascontiguousarray(np.atleast_1d(nu), dtype=np.float64)
        img = A.DeviceImage(*(dev_planes.get(k) for k in PLANES), dev_planes.get("status"))
        check(self.lib, self.lib.jsh_observation_run_device(self.handle, C.byref(model), C.byref(plane),
                                                            A.dptr(nu), nu.size, C.byref(params),
                                                            C.c_void_p(stream_ptr), C.byref(img)))

    def visibilities(self, model: A.ModelDesc, plane: A.PlaneDesc, nu, params: A.Params, uv, rad_per_cm: float,
                     jy_per_cgs: float, dx: float = 0.0, dy: float = 0.0, rot: float = 0.0):
        """Render and transform the Stokes I image on the device
        (jsh_observation_visibilities): ``uv`` [n_uv, 2] wavelengths (the same
        points for every frequency) or [n_nu, n_uv, 2]; returns complex
        visibilities [n_nu, n_uv] in Jy and the render's stats."""
        nu = np.ascontiguousarray(np.atleast_1d(nu), dtype=np.float64)
        uv = np.asarray(uv, dtype=np.float64)
        if uv.ndim == 2:
            uv = np.broadcast_to(uv, (nu.size,) + uv.shape)
        uv = np.ascontiguousarray(uv)
        if uv.shape[0] != nu.size or uv.shape[-1] != 2:
            raise ValueError("uv must be [n_uv, 2] or [n_nu, n_uv, 2]")
        n_uv = uv.shape[1]
        out = np.zeros((nu.size, n_uv, 2))
        vd = A.VisDesc(rad_per_cm=float(rad_per_cm), jy_per_cgs=float(jy_per_cgs), dx=float(dx), dy=float(dy),
                       rot=float(rot))
        st = A.Stats()
        check(self.lib, self.lib.jsh_observation_visibilities(self.handle, C.byref(model), C.byref(plane),
                                                              A.dptr(nu), nu.size, C.byref(params), C.byref(vd),
                                                              A.dptr(uv), n_uv, A.dptr(out), C.byref(st)))
        return out[..., 0] + 1j * out[..., 1], stats_dict(st)

    def autotune(self, model: A.ModelDesc, plane: A.PlaneDesc, nu, params: A.Params) -> dict:
        """Search the persistent schedule's launch shape on this request and
        make the fastest the context default (results do not depend on it)."""
        nu = np.ascontiguousarray(np.atleast_1d(nu), dtype=np.float64)
        t = A.Tuning()
        check(self.lib, self.lib.jsh_autotune(self.handle, C.byref(model), C.byref(plane), A.dptr(nu), nu.size,
                                              C.byref(params), C.byref(t)))
        return {"block_size": t.block_size, "ctas_per_sm": t.ctas_per_sm, "refill_threshold": t.refill_threshold,
                "compact": t.compact, "overlap": t.overlap, "ms": t.ms}

    def last_kernel_ms(self):
        """Device times [ms] of the last request's tau kernel, IQUV ranking and
        IQUV kernel (it must have been enqueued with FLAG_KERNEL_TIMES)."""
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        check(self.lib, self.lib.jsh_last_kernel_ms(self.handle, C.byref(a), C.byref(b), C.byref(c)))
        return {"tau_ms": a.value, "iquv_rank_ms": b.value, "iquv_ms": c.value}

    def last_stats(self):
        st = A.Stats()
        check(self.lib, self.lib.jsh_last_stats(self.handle, C.byref(st)))
        return stats_dict(st)

    def device_peaks(self):
        """Measured FP32 TFLOP/s, MUFU ex2 T ops/s and FP64 TFLOP/s of the device."""
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        check(self.lib, self.lib.jsh_device_peaks(self.handle, C.byref(a), C.byref(b), C.byref(c)))
        return {"fp32_tflops": a.value, "mufu_tops": b.value, "fp64_tflops": c.value}

    # ----------------------------------------------------- inspection
    def plane_rays(self, plane: A.PlaneDesc):
        n = int(plane.n_across * plane.n_along)
        o = np.zeros((n, 3)); d = np.zeros(3); s = np.zeros(n)
        check(self.lib, self.lib.jsh_plane_rays(self.handle, C.byref(plane), A.dptr(o), A.dptr(d), A.dptr(s)))
        return o, d, s

    def trace_plane(self, model: A.ModelDesc, plane: A.PlaneDesc):
        n = int(plane.n_across * plane.n_along)
        nseg = np.zeros(n, np.int32); seg = np.zeros((n, 2, 2, 3)); st = np.zeros(n, np.uint32)
        check(self.lib, self.lib.jsh_trace_plane(self.handle, C.byref(model), C.byref(plane),
                                                 nseg.ctypes.data_as(C.POINTER(C.c_int32)), A.dptr(seg),
                                                 st.ctypes.data_as(C.POINTER(C.c_uint32))))
        return nseg, seg, st

    def hit_rays(self, model: A.ModelDesc, origins, directions):
        origins = np.ascontiguousarray(origins, dtype=np.float64)
        directions = np.ascontiguousarray(directions, dtype=np.float64)
        n = origins.shape[0]
        nseg = np.zeros(n, np.int32); seg = np.zeros((n, 2, 2, 3)); st = np.zeros(n, np.uint32)
        check(self.lib, self.lib.jsh_hit_rays(self.handle, C.byref(model), A.dptr(origins), A.dptr(directions),
                                              n, nseg.ctypes.data_as(C.POINTER(C.c_int32)), A.dptr(seg),
                                              st.ctypes.data_as(C.POINTER(C.c_uint32))))
        return nseg, seg, st

    # ---------------------------------------------------------- gridded fields
    def grid_upload(self, xy, values, tri) -> int:
        """Upload a triangulated (z, r) grid [pc] with per-vertex FP32
        values [n, n_fields]; returns the grid id for Simulation*Field."""
        xy = np.ascontiguousarray(xy, dtype=np.float64)
        values = np.ascontiguousarray(values, dtype=np.float32)
        if values.ndim == 1:
            values = values[:, None]
        tri = np.ascontiguousarray(tri, dtype=np.int32)
        gid = C.c_int32()
        check(self.lib, self.lib.jsh_grid_upload(self.handle, A.dptr(xy), xy.shape[0],
                                                 values.ctypes.data_as(C.POINTER(C.c_float)), values.shape[1],
                                                 tri.ctypes.data_as(C.POINTER(C.c_int32)), tri.shape[0],
                                                 C.byref(gid)))
        return gid.value

    def stripe(self, model: A.ModelDesc, plane: A.PlaneDesc, nu: float, n: int = 100, tau_max: float = 1e4):
        """tau along half of the central row (Observation::run_stripe +
        getStripe) on the device: n_along - n_along // 2 values."""
        out = np.zeros(int(plane.n_along - plane.n_along // 2))
        check(self.lib, self.lib.jsh_observation_run_stripe(self.handle, C.byref(model), C.byref(plane), float(nu),
                                                            int(n), float(tau_max), A.dptr(out)))
        return out

    def hull_upload(self, zr, n_circle: int = 36) -> int:
        """Build and upload the hull of SimulationGeometry: the (z, r) points
        [pc] revolved at n_circle azimuths; returns the hull id."""
        zr = np.ascontiguousarray(zr, dtype=np.float64).reshape(-1, 2)
        hid = C.c_int32()
        check(self.lib, self.lib.jsh_hull_upload(self.handle, A.dptr(zr), zr.shape[0], int(n_circle),
                                                 C.byref(hid)))
        return hid.value

    def cells_upload(self, points, directions) -> int:
        """Upload a random cell set (points [n, 3] cm, unit directions [n, 3])
        for CellsRandomVectorBField; returns its id."""
        p = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        d = np.ascontiguousarray(directions, dtype=np.float64).reshape(-1, 3)
        cid = C.c_int32()
        check(self.lib, self.lib.jsh_cells_upload(self.handle, A.dptr(p), A.dptr(d), p.shape[0], C.byref(cid)))
        return cid.value

    def cells_nearest(self, cells_id: int, points):
        """Nearest cell of each point [n, 3] (cm), found on the device."""
        p = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(p.shape[0], np.int32)
        check(self.lib, self.lib.jsh_cells_nearest(self.handle, cells_id, A.dptr(p), p.shape[0],
                                                   out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    def random_directions(self, seed: int, keys):
        """Random unit directions [n, 3] of the counters keys [n, 3], drawn on the device."""
        k = np.ascontiguousarray(keys, dtype=np.uint32).reshape(-1, 3)
        out = np.zeros((k.shape[0], 3))
        check(self.lib, self.lib.jsh_random_directions(self.handle, int(seed),
                                                       k.ctypes.data_as(C.POINTER(C.c_uint32)), k.shape[0],
                                                       A.dptr(out)))
        return out

    def grid_interpolate(self, grid_id: int, field: int, zr, nan_value=0.0):
        """Values of field `field` at points (z, r) [pc], interpolated on the device."""
        zr = np.ascontiguousarray(zr, dtype=np.float64).reshape(-1, 2)
        out = np.empty(zr.shape[0])
        check(self.lib, self.lib.jsh_grid_interpolate(self.handle, grid_id, field, A.dptr(zr), zr.shape[0],
                                                      float(nan_value), A.dptr(out)))
        return out


def triangulate(xy) -> np.ndarray:
    """Delaunay triangulation of points xy [n, 2] on the host
    (jsh_grid_triangulate): int32 [n_tri, 3], counter-clockwise."""
    lib = A.load_library()
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    tri = np.empty((2 * xy.shape[0], 3), np.int32)
    m = C.c_int64()
    check(lib, lib.jsh_grid_triangulate(A.dptr(xy), xy.shape[0], tri.ctypes.data_as(C.POINTER(C.c_int32)),
                                        C.byref(m)))
    return tri[:m.value].copy()


def cells_generate(n, r_min, r_max, theta_max, exponent, seed):
    """The cells of RandomCellsInSphere on the host (jsh_cells_generate):
    points [n, 3] cm and unit directions [n, 3]."""
    lib = A.load_library()
    p = np.zeros((int(n), 3))
    d = np.zeros((int(n), 3))
    check(lib, lib.jsh_cells_generate(int(n), float(r_min), float(r_max), float(theta_max), float(exponent),
                                      int(seed), A.dptr(p), A.dptr(d)))
    return p, d


def stats_dict(st: A.Stats) -> dict:
    return {f: getattr(st, f) for f, _ in A.Stats._fields_}


_default = None
_lock = threading.Lock()


def default_context() -> Context:
    global _default
    with _lock:
        if _default is None:
            _default = Context(0)
        return _default


def mas_to_pc(z: float, H0=None, omega_M=None, omega_V=None, gamma_nu=None) -> float:
    """Parsecs per mas at redshift z (jsh_mas_to_pc; reference defaults when
    no cosmology is given)."""
    lib = A.load_library()
    if H0 is None:
        return lib.jsh_mas_to_pc(z, None)
    cosmo = A.Cosmology(H0=H0, omega_M=omega_M, omega_V=omega_V, gamma_nu=gamma_nu or 0.0)
    return lib.jsh_mas_to_pc(z, C.byref(cosmo))
