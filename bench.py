"""Benchmark of the full-Stokes transfer path on one GB300.

Workload (one step): the 512 x 1024 log-spaced conical jet at 8.1, 8.4, 12.1
and 15.4 GHz, tau then IQUV at rtol 1e-6 / atol 1e-10, synthetic model of
the configuration (no external data).  The metric counts (hit ray,
frequency) work items per second.

Forms timed in the same run:
  * batched  -- mixed precision (FP32 stages / FP64 tau, Faraday angle and
                step control), persistent refilling schedule: `value`;
  * mixed    -- the same arithmetic, one thread per item (static schedule);
  * batched from tau_max -- the batched form integrating IQUV from tau_max
                like the reference (no optically thick start);
  * plain    -- all-FP64, one thread per item (the plain GPU drop-in).
`e2e` times the batched form through the C ABI with host buffers (outputs
copied back to pinned host memory each step).  Further legs: the 128x128
conical jet (C0), the 1024x1024 ParabaloidCone with a Faraday-thick core
(C2), the simulation-grid jet (C3) and the replayed serving stream (C4).
`--impl reference` times the CPU oracle (FP64 restatement of the
reference's Observation::run with OpenMP over pixels) on bounded samples of
the same workload; it never loads the CUDA library.
"""
from __future__ import annotations

import argparse
import csv
import ctypes as C
import io
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "full_stokes_rays_per_s"
UNIT = "rays/s"
WORKLOAD = ("conical jet 512x1024 log-spaced (lg mas -3..-1), 4 freq (8.1/8.4/12.1/15.4 GHz), full Stokes, "
            "rtol 1e-6 with atol tightened to the 1e-4-qualified tolerances")
# source-level op census of one mixed-precision right-hand-side evaluation
# of this workload's model (ConstFlat V, helical conical B, BK n): FP32
# arithmetic instructions (an FMA counts once) and MUFU ops.  A full-Stokes
# evaluation of the IQUV pass (all coefficients in the log domain, the frame
# rotation, the 4x4 right-hand side; stage combination and error estimate
# amortised over the 6 evaluations of a Dormand-Prince step) and a tau-pass
# evaluation, one node of a Gauss-Kronrod panel (the node's point, k_I only:
# |p|, the helical direction, |n' x u|, two log2, one rsqrt, two exp2; the
# three panel sums)
CENSUS_FP32_INSTR = 116
CENSUS_MUFU = 12
CENSUS_TAU_FP32_INSTR = 34
CENSUS_TAU_MUFU = 5
# DRAM bytes (read + write) per launch of the two transfer kernels of the
# split form, from an ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum) of the 256x512 render (206 368 work items; tau
# kernel 6 537 472 + 1 024 B, IQUV kernel 13 360 384 + 54 272 B) scaled to
# the full render by its work items (826 336)
TRAFFIC_BYTES_PER_LAUNCH = {"transfer_tau_kernel": round((6537472 + 1024) * 826336 / 206368),
                            "transfer_iquv_kernel": round((13360384 + 54272) * 826336 / 206368)}
TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of each transfer kernel on the "
                  "256x512 render, scaled by the hit rays")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scale", type=int, default=1, help="shrink the image (debug only)")
    ap.add_argument("--workload", default="conical", choices=["conical", "simulation-grid"],
                    help="the rendered jet (simulation-grid: profiling of the gridded path only)")
    ap.add_argument("--shape", default="",
                    help="block,ctas_per_sm,refill,compact: fixed launch shape instead of the autotuner "
                         "(profiling: the first persistent launch is then a warm-up step)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-gridded", dest="gridded", action="store_false",
                    help="skip the simulation-grid leg")
    ap.add_argument("--serve-requests", type=int, default=1000,
                    help="requests of the replayed serving stream (0 skips the serving leg)")
    ap.add_argument("--saturate-rate", type=float, default=5000.0,
                    help="arrival rate [1/s] of a second replay that saturates the device (0 skips it)")
    ap.add_argument("--sustain-rate", type=float, default=40.0,
                    help="arrival rate [1/s] of a third replay the device carries (0 skips it)")
    ap.add_argument("--sustain-requests", type=int, default=400,
                    help="requests of the sustainable-rate replay")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="skip the C0 and C2 legs")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(value: float, world: int, device="cuda") -> float:
    """The largest of every rank's value (the slowest replica sets the
    whole job's time); the value itself on one rank."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: int, world: int, ms_per_step_max: float) -> float:
    """Whole-job throughput of replicas: the units all ranks processed in one
    step over the slowest rank's step time."""
    return units_per_rank * world / (ms_per_step_max * 1e-3)


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.rows = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        for row in csv.reader(io.StringIO(out)):
            if len(row) >= 9:
                self.rows.append([x.strip() for x in row])

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def workload(scale, name="conical", ctx=None, pcm=None):
    """The headline workload (the conical jet on the 512x1024 log plane), or
    the simulation-grid jet (its grid triangulated and uploaded to ctx) for
    profiling that path.  ``pcm``: parsecs per mas computed by the caller
    (the reference arm passes the oracle's value)."""
    from jetshow_gb300 import workloads as W
    if name == "simulation-grid":
        from jetshow_gb300.runtime import triangulate
        xy, vals = W.simulation_grid_c3()
        gid = ctx.grid_upload(xy, vals, triangulate(xy))
        return W.simulation_c3(gid, scale=scale)
    return W.conical_c1(scale=scale, pcm=pcm)


def config_dict(image, n_freq, work_items, world):
    """The ``config`` of both arms' lines (the same workload, same keys)."""
    return {"workload": WORKLOAD, "image": list(image), "n_freq": int(n_freq), "work_items": int(work_items),
            "l2": "GPU arm: 256 MB buffer written between timed steps (the CPU reference arm has no device)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def oracle_hits(O, jet, plane):
    """Flat indices of the pixels whose ray hits the jet (the oracle's own
    geometry, bit-exact with the device's)."""
    o, d, _ = O.plane_rays(plane.desc())
    nseg, _, _ = O.hit_rays(jet.desc(), o, np.tile(d, (o.shape[0], 1)))
    return np.nonzero(nseg > 0)[0]


def timed_oracle_sample(O, jet, plane, nu, params, hit, rng, n, threads):
    pix = np.sort(rng.choice(hit, size=min(n, hit.size), replace=False))
    t0 = time.perf_counter()
    O.render(jet.desc(), plane.desc(), nu, params, pix=pix, threads=threads)
    return pix.size * nu.size, time.perf_counter() - t0


def reference_arm(args, step_seconds=2.5):
    """The CPU oracle (OpenMP over pixels on every host core, FP64) on
    bounded random samples of the headline workload: every step renders a
    fresh random sample of hit pixels (all four frequencies) sized during
    the warm-up steps to take about ``step_seconds``.  Only the oracle's
    library is loaded (no CUDA library, no torch)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from jetshow_gb300 import _capi as A
    from jetshow_gb300 import jet as J
    from jetshow_gb300 import workloads as W
    from oracle import oracle as O
    O.build()
    pcm = O.mas_to_pc(W.Z, A.Cosmology(**W.COSMO_FLAT))
    jet, plane, nu, _ = workload(args.scale, pcm=pcm)
    params = J.make_params(**W.ACCURATE_KW)
    threads = O.threads()
    rng = np.random.default_rng(0)
    hit = oracle_hits(O, jet, plane)
    n = min(hit.size, max(64, threads * 16))
    vals, items_total, t_total = [], 0, 0.0
    for step in range(max(args.warmup, 1) + args.steps):
        items, dt = timed_oracle_sample(O, jet, plane, nu, params, hit, rng, n, threads)
        if step >= max(args.warmup, 1):
            vals.append(items / dt)
            items_total += items
            t_total += dt
        else:  # size the sample for about step_seconds per step
            n = int(min(hit.size, max(16, n * step_seconds / max(dt, 1e-3))))
    v = items_total / t_total
    sample = (f"{n} random hit pixels x {nu.size} freq per step (about {step_seconds:.1f} s each), "
              f"{items_total} items in {t_total:.1f} s over {args.steps} steps")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * t_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(plane.image_size, nu.size, hit.size * nu.size, args.gpus), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(jet, plane, nu, kw, seconds=10.0):
    from jetshow_gb300 import jet as J
    from oracle import oracle as O
    O.build()
    params = J.make_params(**kw)
    threads = O.threads()
    hit = oracle_hits(O, jet, plane)
    rng = np.random.default_rng(1)
    n = min(hit.size, max(32, threads * 4))
    total_items, total_t = 0, 0.0
    while total_t < seconds and total_items < hit.size * nu.size:
        items, dt = timed_oracle_sample(O, jet, plane, nu, params, hit, rng, n, threads)
        total_t += dt
        total_items += items
        n = min(hit.size, n * 2)
    return {"value": total_items / total_t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{total_items} (hit pixel, freq) items drawn at random, {total_t:.1f} s"}


def errors_vs_converged(jet, plane, nu, outs, n_pix=2048, extra_pix=None):
    """Worst errors of each form against the converged FP64 oracle
    (rtol 1e-10) on a random sample of hit pixels (every frequency), plus
    ``extra_pix`` (e.g. the deepest pixels): tau relative (rays below
    tau_max), I relative where I > 1e-6 max(I) of the sample, Q/U/V over
    max(I), total flux of the sample."""
    from jetshow_gb300 import jet as J
    from jetshow_gb300 import workloads as W
    from oracle import oracle as O
    O.build()
    ref_status = next(v for v in outs.values() if v is not None)["status"]
    hit = np.nonzero(((ref_status & 1) != 0).any(axis=0))[0]
    pix = np.random.default_rng(7).choice(hit, size=min(n_pix, hit.size), replace=False)
    if extra_pix is not None:
        pix = np.concatenate([pix, np.asarray(extra_pix, dtype=np.int64)])
    pix = np.unique(pix)
    t0 = time.perf_counter()
    ref = O.render(jet.desc(), plane.desc(), nu, J.make_params(**W.CONVERGED_KW), pix=pix, threads=O.threads())
    res = {"sample": f"{pix.size} hit pixels x {nu.size} freq"
                     + (f" (incl. the {len(extra_pix)} deepest)" if extra_pix is not None else "")
                     + f", oracle at rtol 1e-10 ({time.perf_counter() - t0:.1f} s)"}
    for name, out in outs.items():
        if out is None:
            continue
        e = {}
        notx = (ref["tau"] < 1e4) & (out["tau"][:, pix] < 1e4) & ((ref["status"] & 1) != 0)
        e["tau"] = float(np.max(np.abs(out["tau"][:, pix][notx] - ref["tau"][notx]) / np.abs(ref["tau"][notx])))
        for f in range(nu.size):
            Ir, Ig = ref["I"][f], out["I"][f, pix]
            imax = np.abs(Ir).max()
            sel = np.abs(Ir) > 1e-6 * imax
            e["I"] = max(e.get("I", 0.0), float(np.max(np.abs(Ig[sel] - Ir[sel]) / np.abs(Ir[sel]))))
            for k in ("Q", "U", "V"):
                e[k] = max(e.get(k, 0.0), float(np.max(np.abs(out[k][f, pix] - ref[k][f])) / imax))
            e["flux"] = max(e.get("flux", 0.0), float(abs(Ig.sum() - Ir.sum()) / abs(Ir.sum())))
        res[name] = e
    return res


def faraday_depth(jet, plane, nu_hz, pix, n_pts=4000):
    """Faraday depth int k_F dl [rad] along the chord(s) of pixel ``pix``
    with the oracle's lab-frame k_F (src/utils.cpp:77-98 and the thermal
    term), by the trapezoid rule on points clustered geometrically around
    the chord's closest approach to the jet apex (k_F ~ r^-3 there)."""
    from oracle import oracle as O
    o, d, _ = O.plane_rays(plane.desc())
    nseg, seg, _ = O.hit_rays(jet.desc(), o[pix:pix + 1], d[None, :])
    model, nl = jet.desc(), -np.asarray(d)
    total = 0.0
    for k in range(int(nseg[0])):
        a, b = seg[0, k, 0], seg[0, k, 1]
        L = float(np.linalg.norm(b - a))
        u = (b - a) / L
        sc = float(np.clip(-np.dot(a, u), 0.0, L))
        w = L * np.logspace(-10, 0, n_pts)
        s = np.unique(np.clip(np.concatenate([[0.0, L, sc], sc - w, sc + w]), 0.0, L))
        kf = np.array([O.coefficients(model, a + si * u, nl, nu_hz)[4] for si in s])
        total += float(np.sum(0.5 * (kf[1:] + kf[:-1]) * np.diff(s)))
    return total


def serving_leg(ctx, n_requests, rate_hz=200.0, warm=True, flags=0):
    """Replay the seeded Poisson request stream (priors of the model-fitting
    sweep) through the serving loop in real time; latency is arrival to
    result on the host.  ``flags``: JSH_FLAG_* of every request."""
    from jetshow_gb300 import jet as J
    from jetshow_gb300 import serving as S
    from jetshow_gb300 import workloads as W
    stream = S.request_stream(n_requests, rate_hz=rate_hz, seed=42)
    params = J.make_params(precision="mixed", schedule="persistent", flags=flags, **W.ACCURATE_KW)
    counts = {}
    with S.Server(ctx, max_inflight_batches=3, max_batch_requests=16) as srv:
        if warm:  # one short stream first: pages in the result path and the host threads
            S.run_stream(srv, [r for r in S.request_stream(8, rate_hz=200.0, seed=7) if r.size_label == "64x64"],
                         params=params)
        records, wall = S.run_stream(srv, stream, params=params, counts=counts)
    lat = np.array([r["latency_ms"] for r in records])
    queue = np.array([r["queue_ms"] for r in records])
    items = sum(r["n_items"] for r in records)
    by_size = {}
    for label in S.SIZES:
        sel = np.array([r["size"] == label for r in records])
        if sel.any():
            by_size[label] = {"n": int(sel.sum()), "p50_ms": float(np.percentile(lat[sel], 50)),
                              "p99_ms": float(np.percentile(lat[sel], 99))}
    span = stream[-1].t_arrival
    return {"requests": len(stream), "completed": len(records), "arrival_rate_hz": rate_hz, "wall_s": wall,
            "arrival_span_s": span, "rays_per_s": items / wall, "offered_rays_per_s": items / span,
            "work_items": int(items), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "queue_p50_ms": float(np.percentile(queue, 50)), "queue_p99_ms": float(np.percentile(queue, 99)),
            "by_size": by_size, "admission_rejections": int(counts.get("admission_rejections", 0)),
            "mean_batch_requests": float(np.mean([r["batch_size"] for r in records])),
            "tolerances": "rtol 1e-6 / 5e-8 tau, atol 1e-24 / 1e-20 tau, mixed precision, full Stokes"}


def gridded_leg(ctx, steps=3):
    """The simulation-grid jet (203 284-point triangulated grid, 512x512 at
    15.4 GHz, every field interpolated on the device): host triangulation
    and upload time, then the batched and plain forms (device time per
    render)."""
    from jetshow_gb300 import jet as J
    from jetshow_gb300 import workloads as W
    from jetshow_gb300.runtime import triangulate
    t0 = time.perf_counter()
    xy, vals = W.simulation_grid_c3()
    tri = triangulate(xy)
    t1 = time.perf_counter()
    gid = ctx.grid_upload(xy, vals, tri)
    t2 = time.perf_counter()
    out = {"grid_points": int(xy.shape[0]), "triangles": int(tri.shape[0]), "triangulate_s": t1 - t0,
           "upload_s": t2 - t1, "l2": "not flushed: the 13 MB grid is meant to stay resident in the 129 MB L2"}
    # the batched form on the full 512x512 render at the gridded tolerances
    # that meet the accuracy contract (GRID_MIXED_KW) and at the conical
    # jet's (ACCURATE_KW), with the launch shape of the headline's
    # autotuning; the plain FP64 form on a 128x128 render of the same region
    # (its grid lookups are FP64, 1/64 rate) at ACCURATE_KW
    for name, kw, scale, reps, tol in (
            ("batched", dict(precision="mixed", schedule="persistent"), 1, steps, W.GRID_MIXED_KW),
            ("batched_accurate_kw", dict(precision="mixed", schedule="persistent"), 1, steps, W.ACCURATE_KW),
            ("plain_fp64", dict(precision="fp64", schedule="static"), 4, 1, W.ACCURATE_KW)):
        jet, plane, nu, _ = W.simulation_c3(gid, scale=scale)
        p = J.make_params(**kw, **tol)
        ms = []
        for i in range(1 + reps):
            _, st = ctx.render(jet.desc(), plane.desc(), nu, p)
            if i > 0:
                ms.append(st["device_ms"])
            if st["device_ms"] > 20000:  # a bound on the bench's run time
                ms.append(st["device_ms"])
                break
        out[name] = {"rays_per_s": st["n_work_items"] / (np.mean(ms) * 1e-3), "ms": float(np.mean(ms)),
                     "image": list(plane.image_size), "work_items": int(st["n_work_items"]),
                     "rhs_evals": int(st["rhs_evals"]),
                     "tolerances": {k: tol[k] for k in ("tau_rtol", "rtol", "dt_max") if k in tol}}
    return out


class Renderer:
    """Device-timed renders of one workload through jsh_observation_run_device
    into preallocated device planes (CUDA events on the launching stream, a
    256 MB buffer written before every step)."""

    def __init__(self, ctx, torch, max_values):
        self.ctx, self.torch = ctx, torch
        self.stream = torch.cuda.Stream()
        self.planes = {k: torch.zeros(max_values, dtype=torch.float64, device="cuda") for k in
                       ("tau", "l", "I", "Q", "U", "V")}
        self.planes["status"] = torch.zeros(max_values, dtype=torch.int32, device="cuda")
        self.ptrs = {k: v.data_ptr() for k, v in self.planes.items()}
        self.flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(self, model, pdesc, nu, params, steps, warmup, kernel_ms=None):
        """Device time [ms] of each timed step; with ``kernel_ms`` (a list)
        the request's per-kernel times of each timed step are appended to it
        (params carry FLAG_KERNEL_TIMES)."""
        torch = self.torch
        ms = []
        for i in range(warmup + steps):
            self.flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(self.stream):
                e0.record(self.stream)
                self.ctx.render_device(model, pdesc, nu, params, self.stream.cuda_stream, self.ptrs)
                e1.record(self.stream)
            self.stream.synchronize()
            if i >= warmup:
                ms.append(e0.elapsed_time(e1))
                if kernel_ms is not None:
                    kernel_ms.append(self.ctx.last_kernel_ms())
        return ms, self.ctx.last_stats()

    def host(self, n_nu, npix):
        return {k: v[:n_nu * npix].view(n_nu, npix).cpu().numpy() for k, v in self.planes.items()}


def config_leg(R, jet, plane, nu, kw, steps, plain_scale, plain_builder, n_err_pix, n_deep, faraday=False):
    """One more configuration (C0, C2): the batched form on the full image
    (device time), the plain all-FP64 form on the same model at
    ``plain_scale`` (a coarser plane of the same extent: the bounded
    subset), errors of the batched form against the converged oracle on a
    random sample plus the ``n_deep`` deepest pixels, and, when asked, the
    core Faraday depth at the lowest frequency and the batched form with the
    Faraday-thick mode (JSH_FLAG_FARADAY_THICK; its errors on the same
    pixels)."""
    from jetshow_gb300 import jet as J
    from jetshow_gb300 import _capi as A
    model, pdesc = jet.desc(), plane.desc()
    npix = plane.image_size[0] * plane.image_size[1]
    out_f = None
    if faraday:
        ms_f, st_f = R.timed(model, pdesc, nu, J.make_params(precision="mixed", schedule="persistent",
                                                             flags=A.FLAG_FARADAY_THICK, **kw), steps, 1)
        out_f = R.host(nu.size, npix)
    p_b = J.make_params(precision="mixed", schedule="persistent", **kw)
    ms_b, st_b = R.timed(model, pdesc, nu, p_b, steps, 1)
    out_b = R.host(nu.size, npix)
    leg = {"image": list(plane.image_size), "freq_ghz_source": [float(x) / 1e9 for x in nu],
           "work_items": int(st_b["n_work_items"]), "batched": {
               "rays_per_s": st_b["n_work_items"] / (np.mean(ms_b) * 1e-3), "ms": float(np.mean(ms_b)),
               "rhs_evals": int(st_b["rhs_evals"]), "status_or": int(st_b["status_or"])}}
    if faraday:
        leg["batched_faraday_thick_mode"] = {
            "rays_per_s": st_f["n_work_items"] / (np.mean(ms_f) * 1e-3), "ms": float(np.mean(ms_f)),
            "rhs_evals": int(st_f["rhs_evals"]), "status_or": int(st_f["status_or"])}
    jp, plp, nup, _ = plain_builder(plain_scale)
    ms_p, st_p = R.timed(jp.desc(), plp.desc(), nup, J.make_params(precision="fp64", schedule="static", **kw), 1, 0)
    leg["plain_fp64"] = {"rays_per_s": st_p["n_work_items"] / (np.mean(ms_p) * 1e-3), "ms": float(np.mean(ms_p)),
                         "image": list(plp.image_size), "work_items": int(st_p["n_work_items"]),
                         "subset": f"the same model on a {plp.image_size[0]}x{plp.image_size[1]} plane of the same "
                                   f"extent"}
    tau0 = np.where((out_b["status"][0] & 1) != 0, out_b["tau"][0], -1.0)
    deep = np.argsort(tau0)[::-1][:n_deep]
    leg["deepest_tau"] = float(tau0[deep[0]])
    leg["err_vs_converged_oracle"] = errors_vs_converged(jet, plane, nu, {"batched": out_b,
                                                                          "batched_faraday_thick_mode": out_f},
                                                         n_pix=n_err_pix, extra_pix=deep)
    if faraday:
        leg["core_faraday_depth_rad"] = faraday_depth(jet, plane, float(nu[0]), int(deep[0]))
    return leg


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from jetshow_gb300 import jet as J
    from jetshow_gb300 import _capi as A
    from jetshow_gb300 import workloads as W
    from jetshow_gb300.runtime import Context

    ctx = Context(local)
    jet, plane, nu, kw = workload(args.scale, args.workload, ctx)
    model, pdesc = jet.desc(), plane.desc()
    na, nl = plane.image_size
    npix = na * nl
    R = Renderer(ctx, torch, max(nu.size * npix, 2 * 1024 * 1024))

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    kw_cfg = dict(kw)
    kw = dict(W.ACCURATE_KW)  # every form at the 1e-4-qualified tolerances
    p_batched = J.make_params(precision="mixed", schedule="persistent", flags=A.FLAG_KERNEL_TIMES, **kw)
    p_mixed = J.make_params(precision="mixed", schedule="static", **kw)
    p_plain = J.make_params(precision="fp64", schedule="static", **kw)
    p_cfg = J.make_params(precision="mixed", schedule="persistent", **kw_cfg)

    # ---- batched form (headline): the launch shape autotuned on this
    # request (untimed), then clocks sampled during the timed steps
    if args.shape:
        b, c, r, k = (int(x) for x in args.shape.split(","))
        p_batched = J.make_params(precision="mixed", schedule="persistent", block_size=b, ctas_per_sm=c,
                                  refill_threshold=r, flags=A.FLAG_KERNEL_TIMES | (A.FLAG_COMPACT_REGS if k else 0),
                                  **kw)
        tuning = {"block_size": b, "ctas_per_sm": c, "refill_threshold": r, "compact": k, "ms": None,
                  "fixed": True}
    else:
        tuning = ctx.autotune(model, pdesc, nu, p_batched)
    p_tmax = J.make_params(precision="mixed", schedule="persistent", flags=A.FLAG_IQUV_FROM_TAU_MAX, **kw)
    barrier()
    kms = []
    with ClockSampler(local) as clk:
        ms_b, st_b = R.timed(model, pdesc, nu, p_batched, args.steps, args.warmup, kernel_ms=kms)
    barrier()
    # per-kernel device times: the overlapped passes report phases, so the
    # kernels are timed on the serial chain of the same request (untimed for
    # the headline; the same kernels and images)
    p_serial = J.make_params(**{f: getattr(p_batched, f) for f, _ in A.Params._fields_})
    p_serial.flags = int(p_batched.flags) | A.FLAG_SERIAL_PASSES | A.FLAG_KERNEL_TIMES
    kms_serial = []
    ms_s, _ = R.timed(model, pdesc, nu, p_serial, min(args.steps, 10), 2, kernel_ms=kms_serial)
    items = st_b["n_work_items"]
    out_b = R.host(nu.size, npix)
    t_step = max_over_ranks(float(np.mean(ms_b)), world)
    value = job_rate(items, world, t_step)

    # ---- static mixed, configuration tolerances, from tau_max, plain FP64
    ms_m, st_m = R.timed(model, pdesc, nu, p_mixed, min(args.steps, 3), 1)
    mixed_rate = st_m["n_work_items"] / (np.mean(ms_m) * 1e-3)
    ms_c, st_c = R.timed(model, pdesc, nu, p_cfg, min(args.steps, 3), 1)
    cfg_rate = st_c["n_work_items"] / (np.mean(ms_c) * 1e-3)
    ms_t, st_t = R.timed(model, pdesc, nu, p_tmax, min(args.steps, 2), 1)
    tmax_rate = st_t["n_work_items"] / (np.mean(ms_t) * 1e-3)
    out_t = R.host(nu.size, npix)
    plain_rate, out_p = None, None
    if not args.no_plain:
        ms_p, st_p = R.timed(model, pdesc, nu, p_plain, 1, 1)
        plain_rate = st_p["n_work_items"] / (np.mean(ms_p) * 1e-3)
        out_p = R.host(nu.size, npix)
    conical = args.workload == "conical"
    rel = (errors_vs_converged(jet, plane, nu, {"batched": out_b, "batched_from_tau_max": out_t, "plain": out_p})
           if rank == 0 and conical else {})

    # ---- end to end through the C ABI with pinned host buffers
    host = {k: torch.empty((nu.size, npix), dtype=torch.float64, pin_memory=True) for k in
            ("tau", "l", "I", "Q", "U", "V")}
    host["status"] = torch.empty((nu.size, npix), dtype=torch.int32, pin_memory=True)
    img = A.Image(*(C.cast(host[k].data_ptr(), C.POINTER(C.c_double)) for k in ("tau", "l", "I", "Q", "U", "V")),
                  C.cast(host["status"].data_ptr(), C.POINTER(C.c_uint32)))
    st = A.Stats()
    nu_c = np.ascontiguousarray(nu, dtype=np.float64)
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = ctx.lib.jsh_observation_run(ctx.handle, C.byref(model), C.byref(pdesc), A.dptr(nu_c), nu_c.size,
                                         C.byref(p_batched), C.byref(img), C.byref(st))
        t1 = time.perf_counter()
        assert rc == 0, ctx.lib.jsh_last_error()
        if i >= args.warmup:
            e2e_ms.append((t1 - t0) * 1e3)
    e2e_value = job_rate(st.n_work_items, world, max_over_ranks(float(np.mean(e2e_ms)), world))
    d2h = sum(v.numel() * v.element_size() for v in host.values())
    h2d = int(ctx.lib.jsh_request_h2d_bytes(nu_c.size, A.PREC_MIXED))

    # ---- roofline of the dominant kernel: the split form's tau kernel or
    # IQUV kernel, each timed live with CUDA events on the launching stream
    # over the timed steps; the algorithmic work is the source-level census
    # per right-hand-side evaluation times the kernel's evaluations
    peaks = ctx.device_peaks()
    # tau-pass evaluations of a render: the same request with the IQUV pass
    # switched off (tau_min above every depth; the tau pass is unchanged)
    _, st_tau = ctx.render(model, pdesc, nu, J.make_params(precision="mixed", schedule="persistent",
                                                           **dict(kw, tau_min=1e300)))
    n_tau = min(st_tau["rhs_evals"], st_b["rhs_evals"])
    n_iquv = st_b["rhs_evals"] - n_tau
    sec = t_step * 1e-3
    tau_ms = float(np.mean([k["tau_ms"] for k in kms_serial]))
    rank_ms = float(np.mean([k["iquv_rank_ms"] for k in kms_serial]))
    iquv_ms = float(np.mean([k["iquv_ms"] for k in kms_serial]))
    kernels = {}
    for name, n_ev, instr, mufu, ms_k in (("transfer_tau_kernel", n_tau, CENSUS_TAU_FP32_INSTR, CENSUS_TAU_MUFU, tau_ms),
                                          ("transfer_iquv_kernel", n_iquv, CENSUS_FP32_INSTR, CENSUS_MUFU, iquv_ms)):
        ach = n_ev * instr * 2 / (ms_k * 1e-3) / 1e12
        kernels[name] = {"ms": ms_k, "rhs_evals": int(n_ev), "achieved": ach, "frac": ach / peaks["fp32_tflops"],
                         "mufu_frac": n_ev * mufu / (ms_k * 1e-3) / 1e12 / peaks["mufu_tops"],
                         "share_of_serial_step": ms_k / float(np.mean(ms_s))}
    dom = max(kernels, key=lambda k: kernels[k]["ms"])
    evals_per_s = st_b["rhs_evals"] / sec
    fp32_instr = n_tau * CENSUS_TAU_FP32_INSTR + n_iquv * CENSUS_FP32_INSTR
    mufu_ops = n_tau * CENSUS_TAU_MUFU + n_iquv * CENSUS_MUFU
    render_achieved = fp32_instr * 2 / sec / 1e12
    roof = {"bound": "fp32", "kernel": dom, "achieved": kernels[dom]["achieved"], "peak": peaks["fp32_tflops"],
            "unit": "TFLOP/s", "frac": kernels[dom]["frac"], "traffic": TRAFFIC_BYTES_PER_LAUNCH.get(dom),
            "traffic_source": TRAFFIC_SOURCE,
            "peak_source": "measured FMA-chain microbenchmark on this GPU in this run (MEASURED_PEAKS.json "
                           "holds only HBM and bf16 peaks)",
            "kernels": kernels, "iquv_rank_ms": rank_ms,
            "kernel_times": {"source": "the serial chain of the same request (JSH_FLAG_SERIAL_PASSES), CUDA events "
                                       "around each kernel on the launching stream",
                             "serial_ms_per_step": float(np.mean(ms_s)),
                             "overlapped_phases_ms": {k: float(np.mean([d[k] for d in kms]))
                                                      for k in ("tau_ms", "iquv_rank_ms", "iquv_ms")}},
            "render": {"achieved": render_achieved, "frac": render_achieved / peaks["fp32_tflops"],
                       "ms": t_step, "rhs_evals_per_s": evals_per_s,
                       "mufu_frac": mufu_ops / sec / 1e12 / peaks["mufu_tops"]},
            "census": {"fp32_instr_per_rhs": CENSUS_FP32_INSTR, "mufu_per_rhs": CENSUS_MUFU,
                       "fp32_instr_per_tau_rhs": CENSUS_TAU_FP32_INSTR, "mufu_per_tau_rhs": CENSUS_TAU_MUFU,
                       "tau_evals_per_step": int(n_tau), "iquv_evals_per_step": int(n_iquv)},
            "fp64_peak_tflops": peaks["fp64_tflops"]}
    cpu = cpu_baseline_sample(jet, plane, nu, kw) if rank == 0 and conical else None
    serving = saturated = sustained = sustained_ft = None
    if args.serve_requests > 0:
        serving = serving_leg(ctx, args.serve_requests)
        if args.saturate_rate > 0:
            saturated = serving_leg(ctx, args.serve_requests, rate_hz=args.saturate_rate, warm=False)
        if args.sustain_rate > 0 and args.sustain_requests > 0:
            sustained = serving_leg(ctx, args.sustain_requests, rate_hz=args.sustain_rate, warm=False)
            try:  # the same stream, every request with the Faraday-thick mode
                sustained_ft = serving_leg(ctx, args.sustain_requests, rate_hz=args.sustain_rate, warm=False,
                                           flags=A.FLAG_FARADAY_THICK)
            except Exception as e:  # reported, never fatal to the bench line
                sustained_ft = {"error": f"{type(e).__name__}: {e}"}
    gridded = gridded_leg(ctx) if args.gridded else None
    configs = None
    if args.configs and conical and rank == 0:
        configs = {
            "C0": config_leg(R, *W.conical_c0()[:3], kw, 10, 1, lambda s: W.conical_c0(scale=s), 1024, 32),
            "C2": config_leg(R, *W.parabolic_c2()[:3], kw, 2, 32, lambda s: W.parabolic_c2(scale=s), 256, 32,
                             faraday=True)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                "config": config_dict((na, nl), nu.size, items, world),
                "tolerances": {"qualified": {k: W.ACCURATE_KW[k] for k in ("tau_atol", "tau_rtol", "atol", "rtol")},
                               "config": {k: kw_cfg[k] for k in ("tau_atol", "tau_rtol", "atol", "rtol")}},
                "forms": {"batched_rays_per_s": value, "mixed_static_rays_per_s": mixed_rate,
                          "plain_fp64_rays_per_s": plain_rate,
                          "batched_over_plain": (value / plain_rate) if plain_rate else None,
                          "batched_from_tau_max_rays_per_s": tmax_rate,
                          "from_tau_max_over_plain": (tmax_rate / plain_rate) if plain_rate else None,
                          "batched_config_tolerances_rays_per_s": cfg_rate},
                "err_vs_converged_oracle": rel,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "ms_per_step": float(np.mean(e2e_ms))},
                "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary(), "serving": serving,
                "serving_saturated": saturated, "serving_sustainable": sustained,
                "serving_sustainable_faraday_thick": sustained_ft, "gridded": gridded,
                "configs": configs,
                "gpu_launches": int(st_b["kernels_launched"]) * args.steps,
                "gpu_launches_per_step": ({"plane": 2, "hit": 1, "rank": 3, "tau": 2, "iquv_rank": 6, "iquv": 2}
                                          if st_b["kernels_launched"] == 15 else
                                          {"plane": 2, "hit": 1, "rank": 3, "tau": 1, "iquv_rank": 3, "iquv": 1}),
                "autotuned_shape": tuning, "rhs_evals_per_step": st_b["rhs_evals"],
                "steps_accepted": st_b["steps_accepted"], "steps_rejected": st_b["steps_rejected"]}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
