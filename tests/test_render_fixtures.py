"""Committed oracle renders (tests/golden/render_fixtures.npz, written by
tests/golden/make_render_fixtures.py) as regression fixtures: the oracle must
keep reproducing them (CPU), and the GPU's FP64 path must match them within
the contract's gates (GPU)."""
import os
import sys

import numpy as np
import pytest

from helpers import compare_images, flat

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_render_fixtures as M  # noqa: E402

FIX = np.load(os.path.join(HERE, "golden", "render_fixtures.npz"))
NAMES = ["c0_full", "c2_full", "tangled_I"]


def fixture(name):
    return {k: FIX[f"{name}/{k}"] for k in ("tau", "l", "I", "Q", "U", "V", "status")}


def case(name):
    return next(c for c in M.cases() if c[0] == name)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_fixture(oracle, name):
    _, jet, plane, nu, params = case(name)
    r = oracle.render(jet.desc(), plane.desc(), nu, params)
    f = fixture(name)
    assert np.array_equal(r["status"], f["status"])
    for k in ("tau", "l", "I", "Q", "U", "V"):
        np.testing.assert_allclose(r[k], f[k], rtol=1e-10, atol=1e-300, err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_fp64_matches_fixture(ctx, name):
    _, jet, plane, nu, params = case(name)
    g, st = ctx.render(jet.desc(), plane.desc(), nu, params)
    f = fixture(name)
    e = compare_images(flat(g), f, full=name.endswith("full"), tau_max=1e4)
    assert e["n_hit"] == st["n_hit_pixels"] * len(nu) > 0
