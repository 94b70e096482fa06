"""Launch-shape autotuner of the persistent schedule: it returns a valid
shape, and renders under the tuned default are bitwise the renders under
any explicit shape (the shape moves work between lanes, never changes it)."""
import numpy as np
import pytest

from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_autotune_shape_and_invariance(ctx):
    jet, plane, nu, _ = W.conical_c1(scale=16)
    p = J.make_params(precision="mixed", schedule="persistent", **W.ACCURATE_KW)
    explicit = J.make_params(precision="mixed", schedule="persistent", block_size=64, ctas_per_sm=1,
                             refill_threshold=32, **W.ACCURATE_KW)
    before, _ = ctx.render(jet.desc(), plane.desc(), nu, explicit)
    t = ctx.autotune(jet.desc(), plane.desc(), nu, p)
    assert t["block_size"] in (64, 96, 128, 192, 256)
    assert t["ctas_per_sm"] >= 1 and 1 <= t["refill_threshold"] <= 32 and t["ms"] > 0
    assert t["compact"] in (0, 1)
    assert t["overlap"] == 0  # 3 232 work items: too few to overlap the passes
    after, st = ctx.render(jet.desc(), plane.desc(), nu, p)
    assert st["n_work_items"] > 0
    # the register-capped build of the kernel, explicitly
    compact = J.make_params(precision="mixed", schedule="persistent", block_size=96, ctas_per_sm=3,
                            refill_threshold=8, flags=J.A.FLAG_COMPACT_REGS, **W.ACCURATE_KW)
    capped, _ = ctx.render(jet.desc(), plane.desc(), nu, compact)
    for k in ("tau", "I", "Q", "U", "V", "status"):
        assert np.array_equal(before[k], after[k]), k
        assert np.array_equal(before[k], capped[k]), k
