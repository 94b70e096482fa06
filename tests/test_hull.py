"""SimulationGeometry's hull in the oracle (CPU): the closed form used by the
oracle and the device (the n_circle-gon revolution of the upper envelope
of the (z, r) hull) against an independent hull, scipy's Qhull of the
revolved point cloud itself, which is what the reference builds with
CGAL::convex_hull_3 (src/main.cpp:880-897) before intersecting the ray's
line with its faces (src/Geometry.cpp:97-132)."""
import math

import numpy as np
import pytest

from jetshow_gb300 import jet as J

PC = J.pc
HULL_ID = 3


def revolve(zr, n_circle=36):
    """The reference's cloud: (r sin phi_j, r cos phi_j, z), phi_j = j 2 pi / n."""
    ang = np.arange(n_circle) * 2 * math.pi / n_circle
    z = np.repeat(zr[:, 0], n_circle)
    r = np.repeat(zr[:, 1], n_circle)
    a = np.tile(ang, zr.shape[0])
    return np.column_stack([r * np.sin(a), r * np.cos(a), z])


def qhull_clip(cloud, o, d):
    """[t_in, t_out] of the lines o + t d against the hull's facet
    half-spaces (t_in >= t_out on a miss)."""
    from scipy.spatial import ConvexHull
    eq = ConvexHull(cloud).equations  # n . x + off <= 0 inside
    nd = d @ eq[:, :3].T
    no = o @ eq[:, :3].T + eq[:, 3]
    with np.errstate(divide="ignore", invalid="ignore"):
        t = -no / nd
    lo = np.where(nd < 0, t, -np.inf).max(axis=1)
    hi = np.where(nd > 0, t, np.inf).min(axis=1)
    parallel_out = np.any((nd == 0) & (no > 0), axis=1)
    hi = np.where(parallel_out, -np.inf, hi)
    return lo, hi


def profiles():
    rng = np.random.default_rng(11)
    # a rectangular simulation domain (boundary rows and columns + interior)
    zb = np.linspace(0.0, 20.0, 81)
    rb = np.linspace(0.0, 0.5, 21)
    rect = np.vstack([np.column_stack([zb, np.full_like(zb, 0.5)]), np.column_stack([zb, np.zeros_like(zb)]),
                      np.column_stack([np.zeros_like(rb), rb]), np.column_stack([np.full_like(rb, 20.0), rb]),
                      np.column_stack([rng.uniform(0, 20, 500), rng.uniform(0, 0.5, 500)])])
    # a collimating (parabolic) jet boundary: every boundary point is a hull vertex
    zp = np.geomspace(0.01, 20.0, 300)
    para = np.vstack([np.column_stack([zp, 0.1 * np.sqrt(zp)]),
                      np.column_stack([rng.uniform(0.01, 20, 400), rng.uniform(0, 1, 400) * 0.1 * np.sqrt(20)])])
    para = para[para[:, 1] <= 0.1 * np.sqrt(np.maximum(para[:, 0], 1e-12))]
    # a random cloud with a bottom cap at r > 0
    cloud = np.column_stack([rng.uniform(1.0, 5.0, 300), rng.uniform(0.2, 1.0, 300)])
    return {"rectangle": rect, "parabolic": para, "cloud": cloud}


def lines(zr, n, seed):
    """Lines through the hull's neighbourhood in random directions, plus
    image-plane rays at LOS 0.1 (direction (-sin, 0, -cos))."""
    rng = np.random.default_rng(seed)
    zmax, rmax = zr[:, 0].max(), zr[:, 1].max()
    zmin = zr[:, 0].min()
    o = np.column_stack([rng.uniform(-1.3, 1.3, n) * rmax, rng.uniform(-1.3, 1.3, n) * rmax,
                         rng.uniform(zmin - 0.1 * (zmax - zmin), zmax + 0.1 * (zmax - zmin), n)])
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    los = 0.1
    m = n // 2
    d[:m] = (-math.sin(los), 0.0, -math.cos(los))
    return o, d


@pytest.mark.parametrize("name", ["rectangle", "parabolic", "cloud"])
def test_oracle_hull_matches_qhull(oracle, name):
    pytest.importorskip("scipy")
    zr = profiles()[name]
    oracle.hull_register(HULL_ID, zr, 36)
    cloud = revolve(zr, 36)
    o, d = lines(zr, 3000, seed=len(name))
    model = J.Jet(J.SimulationGeometry(HULL_ID), J.ConstFlatVField(10.0), J.RandomScalarBFieldZ(0.1, 1.0),
                  J.BKNFieldZ(500, 2, True)).desc()
    nseg, seg, st = oracle.hit_rays(model, o * PC, d)
    scale = max(zr[:, 0].max(), zr[:, 1].max())
    lo, hi = qhull_clip(cloud, o, d)
    chord = hi - lo
    # chords shorter than 1e-9 of the hull cannot tell hit from tangent
    hit = chord > 1e-9 * scale
    miss = ~(chord > -1e-9 * scale)
    assert hit.sum() > 300 and miss.sum() > 300, (hit.sum(), miss.sum())
    assert np.all(nseg[hit] == 1)
    assert np.all(nseg[miss] == 0)
    # point_in is the end of smaller t
    p_in = o[hit] + lo[hit, None] * d[hit]
    p_out = o[hit] + hi[hit, None] * d[hit]
    np.testing.assert_allclose(seg[hit, 0, 0] / PC, p_in, rtol=0, atol=1e-10 * scale)
    np.testing.assert_allclose(seg[hit, 0, 1] / PC, p_out, rtol=0, atol=1e-10 * scale)


def test_profile_is_upper_envelope(oracle):
    zr = profiles()["parabolic"]
    oracle.hull_register(HULL_ID, zr, 36)
    vz, vr = oracle.hull_profile(HULL_ID)
    assert np.all(np.diff(vz) > 0)
    # every point lies below the envelope; the vertices are input points
    env = np.interp(zr[:, 0], vz, vr)
    assert np.all(zr[:, 1] <= env * (1 + 1e-12) + 1e-15)
    pts = {(float(a), float(b)) for a, b in zr}
    assert all((float(a), float(b)) in pts for a, b in zip(vz, vr))
    # strictly concave (collinear vertices dropped)
    s = np.diff(vr) / np.diff(vz)
    assert np.all(np.diff(s) < 0)


def test_hull_rejects_bad_input(oracle):
    with pytest.raises(RuntimeError):
        oracle.hull_register(HULL_ID, np.array([[1.0, 0.1], [1.0, 0.2]]), 36)  # one z only
    with pytest.raises(RuntimeError):
        oracle.hull_register(HULL_ID, np.array([[1.0, -0.1], [2.0, 0.2]]), 36)  # r < 0
    with pytest.raises(RuntimeError):
        oracle.hull_register(HULL_ID, np.array([[1.0, 0.1], [2.0, 0.2]]), 2)  # n_circle < 3


def product_profile(lib, zr, n_circle=36):
    import ctypes as C
    from jetshow_gb300 import _capi as A
    zr = np.ascontiguousarray(zr, dtype=np.float64)
    vz = np.zeros(zr.shape[0]); vr = np.zeros(zr.shape[0]); m = C.c_int32()
    st = lib.jsh_hull_profile(A.dptr(zr), zr.shape[0], n_circle, A.dptr(vz), A.dptr(vr), C.byref(m))
    return st, vz[:m.value + 1], vr[:m.value + 1]


@pytest.mark.parametrize("name", ["rectangle", "parabolic", "cloud"])
def test_product_profile_equals_oracle(lib, oracle, name):
    """The library's host profile (what jsh_hull_upload puts on the device)
    is bitwise the oracle's, so device and oracle clip against the same
    half-planes."""
    zr = profiles()[name]
    st, vz, vr = product_profile(lib, zr)
    assert st == 0
    oracle.hull_register(HULL_ID, zr, 36)
    oz, orr = oracle.hull_profile(HULL_ID)
    assert np.array_equal(vz, oz) and np.array_equal(vr, orr)


def test_product_profile_rejects_bad_input(lib):
    assert product_profile(lib, np.array([[1.0, 0.1], [1.0, 0.2]]))[0] != 0
    assert product_profile(lib, np.array([[1.0, -0.1], [2.0, 0.2]]))[0] != 0
    assert product_profile(lib, np.array([[1.0, 0.1], [2.0, 0.2]]), n_circle=2)[0] != 0

