"""Host Delaunay triangulation of simulation grids (jsh_grid_triangulate),
no GPU: the triangle set equals Qhull's (scipy) for points in general
position, every edge is locally Delaunay on degenerate lattices, and bad
inputs are rejected."""
import time

import numpy as np
import pytest

from jetshow_gb300 import _capi as A
from jetshow_gb300.runtime import JetshowError, triangulate


def canon(tri):
    t = np.sort(np.asarray(tri), axis=1)
    return set(map(tuple, t.tolist()))


def signed_area(xy, tri):
    a, b, c = xy[tri[:, 0]], xy[tri[:, 1]], xy[tri[:, 2]]
    return (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])


def locally_delaunay_violations(xy, tri, rel=1e-9):
    """Edges whose opposite vertex lies strictly inside the other
    triangle's circumcircle (beyond a relative tolerance)."""
    edges = {}
    for t, (a, b, c) in enumerate(tri.tolist()):
        for u, w, o in ((a, b, c), (b, c, a), (c, a, b)):
            edges[(u, w)] = o
    bad = 0
    for (u, w), o in edges.items():
        q = edges.get((w, u))
        if q is None:
            continue
        pa, pb, pc, pd = xy[u], xy[w], xy[o], xy[q]
        m = np.array([[*(p - pd), np.dot(p - pd, p - pd)] for p in (pa, pb, pc)])
        det = np.linalg.det(m)
        scale = np.abs(m).max() ** 2 * np.abs(m[:, :2]).max()
        if det > rel * scale:
            bad += 1
    return bad


def test_matches_qhull_random():
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(0)
    xy = rng.random((3000, 2)) * [20.0, 0.5]
    tri = triangulate(xy)
    assert np.all(signed_area(xy, tri) > 0)
    assert canon(tri) == canon(spatial.Delaunay(xy).simplices)


def test_matches_qhull_sobol_grid():
    spatial = pytest.importorskip("scipy.spatial")
    qmc = pytest.importorskip("scipy.stats.qmc")
    pts = qmc.Sobol(d=2, scramble=True, seed=0).random_base2(m=14)
    xy = np.column_stack([pts[:, 0] * 20.0, pts[:, 1] * 0.5])
    tri = triangulate(xy)
    assert canon(tri) == canon(spatial.Delaunay(xy).simplices)


def test_lattice_is_locally_delaunay():
    # a square lattice: every cell is co-circular, any diagonal is valid
    g = np.stack(np.meshgrid(np.arange(30.0), np.arange(20.0)), -1).reshape(-1, 2)
    tri = triangulate(g)
    assert np.all(signed_area(g, tri) > 0)
    # 2 triangles per cell
    assert tri.shape[0] == 2 * 29 * 19
    assert locally_delaunay_violations(g, tri) == 0


def test_collinear_hull_points_and_duplicates():
    rng = np.random.default_rng(1)
    inner = rng.random((200, 2)) * 0.8 + 0.1
    border = np.column_stack([np.linspace(0, 1, 11), np.zeros(11)])  # 11 collinear hull points
    xy = np.vstack([inner, border, [[0.0, 1.0], [1.0, 1.0]]])
    tri = triangulate(xy)
    assert np.all(signed_area(xy, tri) > 0)
    used = np.unique(tri)
    assert used.size == xy.shape[0]  # every point is a vertex
    # Euler: n_tri = 2 n - 2 - h (h hull vertices, collinear ones included)
    h = 11 + 2
    assert tri.shape[0] == 2 * xy.shape[0] - 2 - h
    assert locally_delaunay_violations(xy, tri) == 0
    # a duplicated point is merged; the lower index is kept
    dup = np.vstack([xy, xy[5:6]])
    tri2 = triangulate(dup)
    assert canon(tri2) == canon(tri)


def test_rejects_degenerate_input():
    with pytest.raises(JetshowError):
        triangulate(np.column_stack([np.arange(10.0), np.full(10, 0.25)]))  # collinear (an r = const row)
    with pytest.raises(JetshowError):
        triangulate(np.ones((5, 2)))
    with pytest.raises(JetshowError):
        triangulate(np.array([[0.0, 0.0], [1.0, np.nan], [0.0, 1.0]]))
    with pytest.raises(JetshowError) as e:
        triangulate(np.zeros((2, 2)))
    assert e.value.status == A.JSH_ERR_INVALID


def test_full_size_grid_is_fast():
    rng = np.random.default_rng(2)
    xy = rng.random((200_000, 2)) * [20.0, 0.5]
    t0 = time.perf_counter()
    tri = triangulate(xy)
    dt = time.perf_counter() - t0
    # n_tri = 2n - 2 - h with a small hull
    assert 2 * xy.shape[0] - 2 - 200 < tri.shape[0] <= 2 * xy.shape[0] - 5
    assert dt < 10.0
