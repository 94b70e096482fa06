"""Serving loop on the GPU: continuous batching with HBM-budget admission.

* each result is the same rendered alone and in a mix of concurrent
  requests of different sizes and frequency counts (bitwise: an item's
  arithmetic does not depend on which batch, warp or lane runs it), also
  when some requests ask for the Faraday-thick mode (their batches run its
  kernels, the others' the default ones);
* a budget that admits only a few requests at a time still completes every
  request (admission waits for memory to free up);
* a request larger than the whole budget is rejected at submission;
* a queued request can be cancelled;
* a replayed Poisson stream completes with per-request latencies.
"""
import numpy as np
import pytest

from jetshow_gb300 import _capi as A
from jetshow_gb300 import jet as J
from jetshow_gb300 import serving as S
from jetshow_gb300 import workloads as W
from jetshow_gb300.runtime import JetshowError

pytestmark = pytest.mark.gpu

PARAMS = dict(W.ACCURATE_KW)


def small_requests(n=6, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        jet, plane, nu, label = S.sample_request(rng)
        if label in ("64x64", "128x128"):
            out.append((jet, plane, nu))
    return out


def assert_same(a, b):
    for k in ("tau", "I", "Q", "U", "V", "status"):
        assert np.array_equal(a[k], b[k]), k


def test_alone_equals_in_mix(ctx):
    reqs = small_requests()
    p = J.make_params(precision="mixed", schedule="persistent", **PARAMS)
    alone = [ctx.render(j.desc(), pl.desc(), nu, p)[0] for j, pl, nu in reqs]
    with S.Server(ctx, max_inflight_batches=2, max_batch_requests=8) as srv:
        ids = [srv.submit(j.desc(), pl.desc(), nu, p) for j, pl, nu in reqs]
        mixed = [srv.wait(i)[0] for i in ids]
    for a, m in zip(alone, mixed):
        assert_same(a, m)


def test_faraday_thick_requests_alone_equal_in_mix(ctx):
    jet2, plane2, nu2, _ = W.parabolic_c2(scale=4)  # 256x256: Faraday-thick core rays
    reqs = small_requests(4, seed=11)
    p = J.make_params(precision="mixed", schedule="persistent", **PARAMS)
    p_ft = J.make_params(precision="mixed", schedule="persistent", flags=A.FLAG_FARADAY_THICK, **PARAMS)
    mix = [(jet2, plane2, nu2, p_ft), (reqs[0][0], reqs[0][1], reqs[0][2], p), (jet2, plane2, nu2, p),
           (reqs[1][0], reqs[1][1], reqs[1][2], p_ft), (reqs[2][0], reqs[2][1], reqs[2][2], p),
           (reqs[3][0], reqs[3][1], reqs[3][2], p_ft)]
    alone = [ctx.render(j.desc(), pl.desc(), nu, q) for j, pl, nu, q in mix]
    # the mode engages on the ParabaloidCone core: fewer evaluations than the default kernels
    assert alone[0][1]["rhs_evals"] < alone[2][1]["rhs_evals"]
    with S.Server(ctx, max_inflight_batches=2, max_batch_requests=8) as srv:
        ids = [srv.submit(j.desc(), pl.desc(), nu, q) for j, pl, nu, q in mix]
        mixed = [srv.wait(i, timeout_ms=120000)[0] for i in ids]
    for (a, _), m in zip(alone, mixed):
        assert_same(a, m)


def test_budget_admission_queues_and_completes(ctx):
    reqs = small_requests(8, seed=5)
    p = J.make_params(precision="mixed", schedule="persistent", **PARAMS)
    # room for about two 128x128 requests with four frequencies at a time
    budget = 2 * (128 * 128 * (112 + 4 * 52) + (1 << 20))
    with S.Server(ctx, max_inflight_batches=2, max_batch_requests=4, hbm_budget_bytes=budget) as srv:
        ids = [srv.submit(j.desc(), pl.desc(), nu, p) for j, pl, nu in reqs]
        outs = [srv.wait(i, timeout_ms=120000) for i in ids]
    alone = [ctx.render(j.desc(), pl.desc(), nu, p)[0] for j, pl, nu in reqs]
    for (m, st), a in zip(outs, alone):
        assert_same(a, m)
        assert st["latency_ms"] > 0


def test_request_over_budget_is_rejected(ctx):
    jet, plane, nu, _ = W.conical_c1()
    p = J.make_params(precision="mixed", schedule="persistent", **PARAMS)
    with S.Server(ctx, hbm_budget_bytes=64 << 20) as srv:
        with pytest.raises(JetshowError) as e:
            srv.submit(jet.desc(), plane.desc(), nu, p)
        assert e.value.status == A.JSH_ERR_OOM


def test_cancel_queued_request(ctx):
    # one slot, one request per batch: a full-size four-frequency render
    # (about a second of work) keeps the slot busy while the next two queue
    big_jet, big_plane, big_nu, _ = W.conical_c1()
    reqs = [(big_jet, big_plane, big_nu)] + small_requests(2, seed=11)
    p = J.make_params(precision="mixed", schedule="persistent", **PARAMS)
    with S.Server(ctx, max_inflight_batches=1, max_batch_requests=1) as srv:
        ids = [srv.submit(j.desc(), pl.desc(), nu, p) for j, pl, nu in reqs]
        srv.cancel(ids[-1])
        with pytest.raises(JetshowError) as e:
            srv.wait(ids[-1])
        assert e.value.status == A.JSH_ERR_CANCELLED
        for i in ids[:-1]:
            srv.wait(i)


def test_replayed_stream_completes(ctx):
    stream = [r for r in S.request_stream(60, rate_hz=200.0, seed=42) if r.size_label != "512x1024log"][:24]
    with S.Server(ctx, max_inflight_batches=3, max_batch_requests=8) as srv:
        records, wall = S.run_stream(srv, stream)
    assert len(records) == len(stream)
    lat = np.array([r["latency_ms"] for r in records])
    assert np.all(lat > 0) and wall > 0
    assert all(r["status_or"] & A.ST_ERRORS == 0 for r in records)
