"""SimulationGeometry on the GPU (src/Geometry.cpp:92-132): the device's
line / revolved-hull intersection against the oracle's, bit-exact (hit
mask, segment count and every coordinate), on the hull profiles of the CPU
test (whose oracle is checked against Qhull's hull of the revolved cloud),
and a render of the simulation-grid jet bounded by the hull of its own grid
points, the geometry the reference pairs with gridded fields."""
import math

import numpy as np
import pytest

from helpers import compare_images, flat
from jetshow_gb300 import jet as J
from jetshow_gb300 import workloads as W
from jetshow_gb300.runtime import triangulate
from test_hull import lines, profiles

pytestmark = pytest.mark.gpu


def model_of(hull_id):
    return J.Jet(J.SimulationGeometry(hull_id), J.ConstFlatVField(10.0), J.RandomScalarBFieldZ(0.1, 1.0),
                 J.BKNFieldZ(500, 2, True)).desc()


@pytest.mark.parametrize("name", ["rectangle", "parabolic", "cloud"])
def test_hull_hits_bit_exact(ctx, oracle, name):
    zr = profiles()[name]
    hid = ctx.hull_upload(zr, 36)
    oracle.hull_register(hid, zr, 36)
    o, d = lines(zr, 4000, seed=7 + len(name))
    d[:50] = [(math.cos(a), math.sin(a), 0.0) for a in np.linspace(0, 6, 50)]  # lines at constant z
    o *= J.pc
    n1, s1, t1 = ctx.hit_rays(model_of(hid), o, d)
    n2, s2, t2 = oracle.hit_rays(model_of(hid), o, d)
    assert np.array_equal(n1, n2)
    assert np.array_equal(t1, t2)
    assert np.array_equal(s1, s2)
    assert (n1 == 1).sum() > 500


def test_hull_plane_bit_exact(ctx, oracle):
    zr = profiles()["parabolic"]
    hid = ctx.hull_upload(zr, 36)
    oracle.hull_register(hid, zr, 36)
    lg = math.log10(0.02 * 1.8443 * J.pc)
    for pl in (J.ImagePlane((64, 96), lg, lg, 0.1), J.ImagePlane((32, 64), lg - 1.5, lg + 0.5, 0.3)):
        o, d, _ = oracle.plane_rays(pl.desc())
        n1, s1, t1 = ctx.trace_plane(model_of(hid), pl.desc())
        n2, s2, t2 = oracle.hit_rays(model_of(hid), o, np.tile(d, (o.shape[0], 1)))
        assert np.array_equal(n1, n2)
        assert np.array_equal(s1[n1 > 0, 0], s2[n2 > 0, 0])
        assert (n1 > 0).sum() > 100


def test_unknown_hull_is_an_error(ctx):
    with pytest.raises(Exception):
        ctx.hit_rays(model_of(15), np.zeros((1, 3)), np.array([[0.0, 0.0, 1.0]]))


def test_simulation_jet_in_its_hull_vs_oracle(ctx, oracle):
    """Every field from the 200k-point simulation grid and the jet bounded by
    the hull of its points with z in [0.5, 19.5] pc and r <= 0.45 pc (a
    36-gon prism inside the grid's rectangle): the batched form at the
    gridded-field tolerances against the converged oracle, at the contract
    gates (the FP64 device path on a hull-bounded grid jet is checked
    against the oracle in test_gpu_grid.py).  The hull of all the grid points
    would put the chords' end points on the grid's own boundary, where
    rounding lands some of them a hair outside: there B = nan_value = 0 and
    the reference's cos(theta) = B.n / |B| of k_V and k_F is 0/0, a NaN that
    the FP64 path reproduces (status JSH_ST_NAN) and the mixed path's folded
    algebra does not."""
    xy, vals = W.simulation_grid_c3()
    tri = triangulate(xy)
    gid = ctx.grid_upload(xy, vals, tri)
    oracle.grid_register(gid, xy, vals, tri)
    inner = xy[(xy[:, 0] >= 0.5) & (xy[:, 0] <= 19.5) & (xy[:, 1] <= 0.45)]
    hid = ctx.hull_upload(inner, 36)
    oracle.hull_register(hid, inner, 36)
    jet, plane, nu, _ = W.simulation_c3(gid, scale=32)
    jet.geometry = J.SimulationGeometry(hid)
    gm, st = ctx.render(jet.desc(), plane.desc(), nu,
                        J.make_params(precision="mixed", schedule="persistent", **W.GRID_MIXED_KW))
    rc = oracle.render(jet.desc(), plane.desc(), nu, J.make_params(**W.GRID_CONVERGED_KW))
    e = compare_images(flat(gm), rc, full=True, tau_max=1e4)
    assert e["n_hit"] == st["n_hit_pixels"] > 0
