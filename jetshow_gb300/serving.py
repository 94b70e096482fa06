"""Python client of the serving loop (``jsh_server_*`` in the C ABI) and the
synthetic request stream of the model-fitting serving benchmark.

The stream: Poisson arrivals (mean rate 200 requests/s by default) of
renders with parameters drawn from seeded priors -- LOS angle U(0.02, 0.3)
rad, cone half-angle U(0.01, 0.1) rad, B0 log-U(0.01, 1) G, n0
log-U(10, 1e4) cm^-3, Gamma U(2, 20); Cone or ParabaloidCone with equal
probability; image 64^2, 128^2, 256^2 or 512x1024 log-spaced; 1-4
frequencies log-uniform in 5-43 GHz.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np

from . import _capi as A
from . import jet as J
from .runtime import PLANES, Context, check, default_context
from .workloads import ACCURATE_KW, Z, _lg_cm


class Server:
    """A ``jsh_server`` on a context: submit renders, wait for results."""

    def __init__(self, ctx: Context | None = None, max_inflight_batches=3, max_batch_requests=16,
                 precision="mixed", use_graphs=True, hbm_budget_bytes=0):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        cfg = A.ServerConfig(max_inflight_batches=max_inflight_batches, max_batch_requests=max_batch_requests,
                             precision={"mixed": A.PREC_MIXED, "fp64": A.PREC_FP64}[precision],
                             use_graphs=int(use_graphs), hbm_budget_bytes=hbm_budget_bytes)
        h = C.c_void_p()
        check(self.lib, self.lib.jsh_server_create(self.ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h
        self.precision = precision
        self._shapes = {}

    def close(self):
        if self.handle:
            self.lib.jsh_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, model: A.ModelDesc, plane: A.PlaneDesc, nu, params: A.Params) -> int:
        nu = np.ascontiguousarray(np.atleast_1d(nu), dtype=np.float64)
        rid = C.c_uint64()
        check(self.lib, self.lib.jsh_server_submit(self.handle, C.byref(model), C.byref(plane), A.dptr(nu), nu.size,
                                                   C.byref(params), C.byref(rid)))
        self._shapes[rid.value] = (nu.size, int(plane.n_across), int(plane.n_along))
        return rid.value

    def poll(self, rid: int) -> bool:
        st = self.lib.jsh_server_poll(self.handle, rid)
        if st < 0:
            check(self.lib, st)
        return st == 1

    def cancel(self, rid: int):
        check(self.lib, self.lib.jsh_server_cancel(self.handle, rid))

    def wait(self, rid: int, timeout_ms: int = -1, want=PLANES):
        n_nu, na, nl = self._shapes.pop(rid)
        out = {k: np.zeros((n_nu, na, nl)) for k in want}
        out["status"] = np.zeros((n_nu, na, nl), np.uint32)
        img = A.Image(*(A.dptr(out[k]) if k in out else None for k in PLANES),
                      out["status"].ctypes.data_as(C.POINTER(C.c_uint32)))
        st = A.RequestStats()
        check(self.lib, self.lib.jsh_server_wait(self.handle, rid, timeout_ms, C.byref(img), C.byref(st)))
        return out, {f: getattr(st, f) for f, _ in A.RequestStats._fields_}


@dataclass
class StreamRequest:
    t_arrival: float  # s from the start of the stream
    jet: J.Jet
    plane: J.ImagePlane
    nu: np.ndarray
    size_label: str


SIZES = ("64x64", "128x128", "256x256", "512x1024log")


def sample_request(rng: np.random.Generator) -> tuple:
    los = rng.uniform(0.02, 0.3)
    half = rng.uniform(0.01, 0.1)
    b0 = 10 ** rng.uniform(-2, 0)
    n0 = 10 ** rng.uniform(1, 4)
    gamma = rng.uniform(2, 20)
    if rng.random() < 0.5:
        geo = J.Cone((0, 0, 0), (0, 0, 1), half, 100.0 * J.pc)
    else:
        # a ParabaloidCone whose tangent cone at the break has the drawn half-angle
        z0 = 1.0 * J.pc
        r0 = 2.0 * math.tan(half) * math.sqrt(z0 * J.pc)
        geo = J.ParabaloidCone((0, 0, 0), (0, 0, 1), r0, z0, 100.0 * J.pc)
    jet = J.Jet(geo, J.ConstFlatVField(gamma), J.HelicalConicalBField(b0, 1.0, math.pi / 4, True),
                J.BKNField(n0, 2.0, True), s=2.5, gamma_min=10.0)
    label = SIZES[int(rng.integers(0, 4))]
    if label == "512x1024log":
        plane = J.ImagePlane((512, 1024), _lg_cm(1e-3), _lg_cm(1e-1), los)
    else:
        n = int(label.split("x")[0])
        mas = 0.1 * 128 / n
        plane = J.ImagePlane((n, n), _lg_cm(mas), _lg_cm(mas), los)
    n_nu = int(rng.integers(1, 5))
    nu = np.sort(10 ** rng.uniform(math.log10(5e9), math.log10(43e9), n_nu)) * (1 + Z)
    return jet, plane, nu, label


def request_stream(n: int, rate_hz: float = 200.0, seed: int = 42) -> list:
    """n requests with exponential inter-arrival times (Poisson process)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(n):
        t += rng.exponential(1.0 / rate_hz)
        jet, plane, nu, label = sample_request(rng)
        out.append(StreamRequest(t, jet, plane, nu, label))
    return out


def run_stream(server: Server, stream: list, params: A.Params | None = None, keep_results=False,
               counts: dict | None = None):
    """Replay a request stream in real time: submit each request at its
    arrival time while a collector thread copies every finished result to
    the host as soon as it completes (in completion order).  Returns the
    per-request records (``latency_ms`` = scheduled arrival to result on
    host, so a late submission counts against the server) and the wall time
    of the whole stream.  A request the server refuses at admission (larger
    than its whole HBM budget: ``JSH_ERR_OOM``) is counted, not raised;
    ``counts`` (if given) receives ``submitted`` and ``admission_rejections``."""
    from .runtime import JetshowError
    import threading

    params = params or J.make_params(precision=server.precision, schedule="persistent", **ACCURATE_KW)
    pending = {}
    lock = threading.Lock()
    records = []
    done_submitting = threading.Event()
    errors = []

    def collect():
        while True:
            with lock:
                items = list(pending.items())
            if not items and done_submitting.is_set():
                return
            progressed = False
            for rid, r in items:
                try:
                    if not server.poll(rid):
                        continue
                    img, st = server.wait(rid, timeout_ms=0, want=("I",) if not keep_results else PLANES)
                except Exception as e:  # noqa: BLE001 - reported to the caller
                    errors.append(e)
                    with lock:
                        pending.pop(rid, None)
                    continue
                st["latency_ms"] = (time.perf_counter() - t0 - r.t_arrival) * 1e3
                st["size"] = r.size_label
                st["n_items"] = int(((img["status"] & A.ST_HIT) != 0).sum())
                if keep_results:
                    st["image"] = img
                    st["request"] = r
                records.append(st)
                with lock:
                    pending.pop(rid, None)
                progressed = True
            if not progressed:
                time.sleep(0.0002)

    th = threading.Thread(target=collect, daemon=True)
    rejected = 0
    t0 = time.perf_counter()
    th.start()
    try:
        for r in stream:
            now = time.perf_counter() - t0
            if r.t_arrival > now:
                time.sleep(r.t_arrival - now)
            try:
                rid = server.submit(r.jet.desc(), r.plane.desc(), r.nu, params)
            except JetshowError as e:
                if e.status != A.JSH_ERR_OOM:
                    raise
                rejected += 1
                continue
            with lock:
                pending[rid] = r
    finally:
        done_submitting.set()
        th.join()
    wall = time.perf_counter() - t0
    if counts is not None:
        counts["submitted"] = len(stream) - rejected
        counts["admission_rejections"] = rejected
    if errors:
        raise errors[0]
    return records, wall
