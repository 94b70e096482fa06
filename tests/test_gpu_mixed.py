"""GPU parity of the mixed-precision path (FP32 right-hand sides and stages,
FP64 tau / Faraday angle / step control) in both schedules against the FP64
oracle at the same tolerances, with the contract's gates."""
import numpy as np
import pytest

from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W
from helpers import compare_images, flat

pytestmark = pytest.mark.gpu

SCHEDULES = ["static", "persistent"]


def run(ctx, oracle, jet, plane, nu, schedule, **kw):
    p_ref = J.make_params(**kw)
    p = J.make_params(precision="mixed", schedule=schedule, **kw)
    g, st = ctx.render(jet.desc(), plane.desc(), nu, p)
    r = oracle.render(jet.desc(), plane.desc(), nu, p_ref)
    return flat(g), r, st


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("output", ["I", "full"])
def test_mixed_conical_c0(ctx, oracle, schedule, output):
    jet, plane, nu, kw = W.conical_c0(scale=4)
    kw["output"] = output
    g, r, st = run(ctx, oracle, jet, plane, nu, schedule, **kw)
    e = compare_images(g, r, full=(output == "full"), tau_max=kw["tau_max"])
    assert st["rhs_evals"] > 0 and st["n_work_items"] == e["n_hit"]


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_mixed_log_plane_multifreq(ctx, oracle, schedule):
    jet, plane, nu, kw = W.conical_c1(scale=16)
    g, r, st = run(ctx, oracle, jet, plane, nu, schedule, **kw)
    compare_images(g, r, full=True, tau_max=kw["tau_max"])


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_mixed_parabolic_faraday(ctx, oracle, schedule):
    jet, plane, nu, kw = W.parabolic_c2(scale=32)
    g, r, st = run(ctx, oracle, jet, plane, nu, schedule, **kw)
    compare_images(g, r, full=True, tau_max=kw["tau_max"])


def test_mixed_tangled_reference_model(ctx, oracle):
    import math
    jet = J.Jet(J.Cone((0., 0., 0.), (0., 0., 1.), 0.0165, 100), J.ConstCentralVField(8.0),
                J.RandomScalarBFieldZ(0.1, 1.0), J.BKNFieldZ(500, 2, True), s=3.42)
    plane = J.ImagePlane((12, 20), math.log10(1e-2 * 1.86 * J.pc), math.log10(1e-1 * 1.86 * J.pc), 0.05)
    g, r, st = run(ctx, oracle, jet, plane, [15.4e9 * 1.1], "persistent", output="I")
    compare_images(g, r, full=False, tau_max=1e4)


@pytest.mark.parametrize("refill", [1, 8, 32])
def test_persistent_refill_thresholds_agree(ctx, refill):
    jet, plane, nu, kw = W.conical_c1(scale=16)
    base = J.make_params(precision="mixed", schedule="static", **kw)
    a, _ = ctx.render(jet.desc(), plane.desc(), nu, base)
    p = J.make_params(precision="mixed", schedule="persistent", refill_threshold=refill, block_size=64, **kw)
    b, _ = ctx.render(jet.desc(), plane.desc(), nu, p)
    # the same per-item arithmetic whichever lane or warp runs an item
    for k in ("tau", "I", "Q", "U", "V", "status"):
        assert np.array_equal(a[k], b[k]), k
