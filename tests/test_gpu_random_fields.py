"""Random vector B fields on the GPU (RandomVectorBField and its cell and
per-evaluation kinds, src/BField.cpp:149-193) against the oracle.

* Draws: the device's random unit directions equal the oracle's bit for bit.
* Cells: the device's nearest cell (bucket grid, exact FP64 distances)
  equals the oracle's scan of every cell, inside and outside the grid.
* CellsRandomVectorBField renders: FP64 device against the oracle at tight
  tolerances (B jumps across the faces between cells), mixed precision
  against the converged oracle; contract gates.
* PointsRandomVectorBField renders are deterministic: the same image twice,
  from the static and the persistent schedule (the draw is keyed by pixel,
  frequency and evaluation index, not by the lane or thread that runs it).
"""
import math

import numpy as np
import pytest

from jetshow_gb300 import _capi as A
from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W
from helpers import compare_images, flat

pytestmark = pytest.mark.gpu

PC = J.pc
TIGHT_KW = dict(W.ACCURATE_KW, tau_rtol=1e-11, rtol=1e-10)


@pytest.fixture(scope="module")
def cells(ctx, oracle):
    c = J.RandomCellsInSphere(400, 2.0, seed=21)
    c.setGeometry(40 * PC, 0.12)
    c.create()
    c.upload(ctx)
    oracle.cells_register(c.id, c.points, c.directions)
    return c


def model(bfield):
    jet = W.conical_model()
    jet.bfield = bfield
    pcm = W.pc_per_mas()
    plane = J.ImagePlane((12, 20), math.log10(10 ** -2.5 * pcm * PC), math.log10(10 ** -0.5 * pcm * PC), 0.1)
    return jet, plane, np.array([8.4e9, 15.4e9]) * (1 + W.Z)


def test_random_directions_bitwise(ctx, oracle):
    rng = np.random.default_rng(2)
    keys = rng.integers(0, 2 ** 32, size=(5000, 3), dtype=np.uint64).astype(np.uint32)
    for seed in (0, 12345, 2 ** 63 + 7):
        assert np.array_equal(ctx.random_directions(seed, keys), oracle.random_directions(seed, keys))


def test_nearest_cell_bitwise(ctx, oracle, cells):
    rng = np.random.default_rng(3)
    q = np.vstack([cells.points[:200] + rng.normal(scale=0.01 * PC, size=(200, 3)),
                   rng.uniform(-10 * PC, 10 * PC, size=(3000, 3)) + [0, 0, 20 * PC],
                   rng.uniform(-200 * PC, 200 * PC, size=(1000, 3)),   # far outside the grid
                   cells.points[:50]])                                # on the points themselves
    got = ctx.cells_nearest(cells.id, q)
    assert np.array_equal(got, oracle.cells_nearest(cells.id, q))
    assert np.array_equal(got[-50:], np.arange(50))


def test_cells_random_field_fp64_vs_oracle(ctx, oracle, cells):
    jet, plane, nu = model(J.CellsRandomVectorBField(cells, J.HelicalConicalBField(0.1, 1.0, math.pi / 4, False), 0.5))
    p = J.make_params(precision="fp64", schedule="static", **TIGHT_KW)
    g, st = ctx.render(jet.desc(), plane.desc(), nu, p)
    r = oracle.render(jet.desc(), plane.desc(), nu, p)
    e = compare_images(flat(g), r, full=True, tau_max=1e4)
    assert e["n_hit"] > 50


def test_cells_random_field_mixed_vs_converged(ctx, oracle, cells):
    # the field jumps across every face between cells (a few hundred faces
    # along a ray), where the Dormand-Prince tau pass converges slowly: at
    # tau_rtol 5e-8 the worst tau is 1.2e-5 .. 1.6e-5 off the converged
    # oracle with steps of at most 0.01 or 0.003 pc, in FP64 on the device
    # as well (1.5e-5 .. 1.7e-5: the reference's algorithm at that
    # tolerance); tau_rtol 1e-9 with 0.003 pc steps gives 1.2e-6
    jet, plane, nu = model(J.CellsRandomVectorBField(cells, J.HelicalConicalBField(0.1, 1.0, math.pi / 4, False), 0.5))
    kw = dict(W.ACCURATE_KW, rtol=1e-7, tau_rtol=1e-9, dt_max=0.003 * PC)
    g, st = ctx.render(jet.desc(), plane.desc(), nu, J.make_params(precision="mixed", schedule="persistent", **kw))
    r = oracle.render(jet.desc(), plane.desc(), nu, J.make_params(**W.CONVERGED_KW))
    compare_images(flat(g), r, full=True, tau_max=1e4)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_points_random_field_is_deterministic(ctx, precision):
    jet, plane, nu = model(J.PointsRandomVectorBField(J.HelicalConicalBField(0.1, 1.0, math.pi / 4, True), 0.05,
                                                      seed=77))
    # a fresh direction at every evaluation makes the right-hand side noise:
    # the adaptive steps shrink until max_steps (as they would in the
    # reference); the test bounds them and checks the determinism
    kw = dict(W.ACCURATE_KW, max_steps=3000)
    a, sa = ctx.render(jet.desc(), plane.desc(), nu, J.make_params(precision=precision, schedule="static", **kw))
    b, sb = ctx.render(jet.desc(), plane.desc(), nu, J.make_params(precision=precision, schedule="persistent", **kw))
    c, _ = ctx.render(jet.desc(), plane.desc(), nu, J.make_params(precision=precision, schedule="persistent", **kw))
    for k in ("tau", "I", "Q", "U", "V", "status"):
        assert np.array_equal(a[k], b[k]) and np.array_equal(b[k], c[k]), k
    assert sa["rhs_evals"] == sb["rhs_evals"]
    hit = (a["status"] & A.ST_HIT) != 0
    assert hit.sum() > 50 and np.isfinite(a["I"][hit]).all()
    assert ((a["status"][hit] & A.ST_STEP_LIMIT) != 0).any()
