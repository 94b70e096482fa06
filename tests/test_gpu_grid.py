"""Gridded (simulation) fields on the GPU: device interpolation against the
oracle's, a linear known answer, and the 200k-point simulation-grid render
against the oracle (FP64) and against the converged oracle (mixed)."""
import numpy as np
import pytest

from helpers import compare_images, flat
from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W
from jetshow_gb300.runtime import triangulate

pytestmark = pytest.mark.gpu

NAN = -7.0


@pytest.fixture(scope="module")
def c3(ctx, oracle):
    xy, vals = W.simulation_grid_c3()
    tri = triangulate(xy)
    gid = ctx.grid_upload(xy, vals, tri)
    oracle.grid_register(gid, xy, vals, tri)
    return gid, xy, vals, tri


def test_interpolation_matches_oracle(ctx, oracle, c3):
    """Device point location and barycentric value against the oracle's,
    bit for bit (src/SimulationInterpolater.cpp:43-102), at random points in
    and outside the grid and at its vertices."""
    gid, xy, vals, tri = c3
    rng = np.random.default_rng(5)
    q = np.column_stack([rng.uniform(-1.0, 21.0, 20000), rng.uniform(-0.05, 0.55, 20000)])
    q = np.vstack([q, xy[:2000]])  # and the vertices themselves
    for field in range(vals.shape[1]):
        g = ctx.grid_interpolate(gid, field, q, nan_value=NAN)
        r = np.array([oracle.grid_value(gid, field, z, rr, NAN) for z, rr in q])
        # the same rounding order on both sides: the same triangle, the same bits
        assert np.array_equal(g, r), field
        assert (r != NAN).sum() > 15000
        # at a vertex the interpolant is the vertex's FP32 value
        np.testing.assert_allclose(g[-2000:], vals[:2000, field].astype(np.float64), rtol=1e-12)


def test_interpolation_reproduces_linear_field(ctx):
    rng = np.random.default_rng(9)
    xy = rng.random((5000, 2)) * [20.0, 0.5]
    xy[:4] = [[0, 0], [20, 0], [0, 0.5], [20, 0.5]]  # the hull is the rectangle
    f = (1.0 + 0.5 * xy[:, 0] + 2.0 * xy[:, 1]).astype(np.float32)
    gid = ctx.grid_upload(xy, f, triangulate(xy))
    q = rng.random((10000, 2)) * [20.0, 0.5]
    g = ctx.grid_interpolate(gid, 0, q, nan_value=NAN)
    exact = 1.0 + 0.5 * q[:, 0] + 2.0 * q[:, 1]
    np.testing.assert_allclose(g, exact, rtol=2e-7)  # FP32 vertex values
    out = ctx.grid_interpolate(gid, 0, [[-1.0, 0.2], [10.0, 0.6], [21.0, 0.1]], nan_value=NAN)
    assert np.all(out == NAN)


# The interpolated fields have kinks at every triangle edge.  Two
# implementations of the same FP64 algorithm are compared at GRID_TIGHT_KW
# (a last-bit difference moves the adaptive steps across the kinks; at these
# tolerances the two images stay within 1e-6 of each other), on a short jet
# bounded by the hull of the grid points with 1 <= z <= 2 pc and r <= 0.1 pc
# (one thread per item on the FP64 pipe, the lanes of a warp diverging: the
# heaviest ray sets the test's time).  The mixed path is compared with a converged solution at
# GRID_MIXED_KW.  Every gate is the contract's.


def short_jet(ctx, oracle, c3, scale):
    gid, xy, _, _ = c3
    inner = xy[(xy[:, 0] >= 1.0) & (xy[:, 0] <= 2.0) & (xy[:, 1] <= 0.1)]
    hid = ctx.hull_upload(inner, 36)
    oracle.hull_register(hid, inner, 36)
    jet, plane, nu, _ = W.simulation_c3(gid, scale=scale)
    jet.geometry = J.SimulationGeometry(hid)
    return jet, plane, nu


def test_fp64_simulation_render_vs_oracle(ctx, oracle, c3):
    jet, plane, nu = short_jet(ctx, oracle, c3, 64)
    p = J.make_params(precision="fp64", schedule="static", **W.GRID_TIGHT_KW)
    g, st = ctx.render(jet.desc(), plane.desc(), nu, p)
    r = oracle.render(jet.desc(), plane.desc(), nu, p)
    e = compare_images(flat(g), r, full=True, tau_max=1e4)
    assert e["n_hit"] == st["n_hit_pixels"] > 0
    assert np.abs(r["I"]).max() > 0


def test_mixed_simulation_render_vs_converged(ctx, oracle, c3):
    gid = c3[0]
    jet, plane, nu, _ = W.simulation_c3(gid, scale=16)
    g, st = ctx.render(jet.desc(), plane.desc(), nu,
                       J.make_params(precision="mixed", schedule="persistent", **W.GRID_MIXED_KW))
    r = oracle.render(jet.desc(), plane.desc(), nu, J.make_params(**W.GRID_CONVERGED_KW))
    compare_images(flat(g), r, full=True, tau_max=1e4)
