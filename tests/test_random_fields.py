"""Random vector B fields on the host: the counter-based generator and the
cells of RandomCellsInSphere (no GPU).

* The oracle's Philox4x32-10 reproduces the published known-answer vectors
  of Salmon et al. (SC'11, the Random123 distribution's kat_vectors).
* The library's host generation of cells (jsh_cells_generate) equals the
  oracle's restatement bit for bit: positions (generate_random_points_sphere,
  src/utils.cpp:267-312) and directions (generate_random_directions,
  src/utils.cpp:249-261).
* The reference's quirk with an unrestricted polar angle (theta_max = 0
  gives cos(theta) = 1 for every point: all cells on the +z axis) is kept.
"""
import math

import numpy as np
import pytest

from jetshow_gb300 import _capi as A
from jetshow_gb300 import jet as J
from jetshow_gb300.runtime import cells_generate

KAT = [  # counter, key (k1 << 32 | k0), output
    ([0, 0, 0, 0], 0, [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, 0xffffffffffffffff, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], (0x299f31d0 << 32) | 0xa4093822,
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
]


def test_philox_known_answers(oracle):
    for ctr, key, out in KAT:
        assert oracle.philox4x32(ctr, key) == out


@pytest.mark.parametrize("args", [(1000, 0.0, 10 * J.pc, 0.1, 2.0, 42), (500, 1 * J.pc, 20 * J.pc, 0.05, 2.0, 7),
                                  (300, 0.0, 3.0, 0.3, 1.5, 1)])
def test_cells_generate_matches_oracle(lib, oracle, args):
    p, d = cells_generate(*args)
    po, do = oracle.cells_generate(*args)
    assert np.array_equal(p, po) and np.array_equal(d, do)
    assert np.all(np.abs(np.linalg.norm(d, axis=1) - 1.0) < 4e-16)
    r = np.linalg.norm(p, axis=1)
    n, r_min, r_max, theta_max, expo, _ = args
    if expo == 2.0:  # r = r^(1/(3-2)) is uniform in [r_min, r_max]
        assert r.min() >= r_min * (1 - 1e-12) and r.max() <= r_max * (1 + 1e-12)
    cos_t = np.abs(p[:, 2]) / r
    assert np.all(cos_t >= math.cos(theta_max) - 1e-12)  # inside the two cones


def test_directions_are_isotropic(oracle):
    keys = np.column_stack([np.arange(20000), np.full(20000, 3), np.full(20000, 11)])
    d = oracle.random_directions(5, keys)
    assert np.all(np.abs(np.linalg.norm(d, axis=1) - 1) < 4e-16)
    assert np.all(np.abs(d.mean(axis=0)) < 0.02)
    assert np.allclose((d ** 2).mean(axis=0), 1 / 3, atol=0.01)


def test_unrestricted_polar_angle_quirk(lib):
    p, _ = cells_generate(50, 0.0, 5.0, 0.0, 2.0, 3)
    assert np.all(p[:, 0] == 0) and np.all(p[:, 1] == 0) and np.all(p[:, 2] >= 0)


def test_random_field_descriptors():
    b = J.HelicalConicalBField(0.1, 1.0, math.pi / 4, False)
    cells = J.RandomCellsInSphere(10, 2.0, seed=4)
    cells.id = 3
    jet = J.Jet(J.Cone((0, 0, 0), (0, 0, 1), 0.05, 1e20), J.ConstFlatVField(10.0),
                J.CellsRandomVectorBField(cells, b, 0.5), J.BKNField(500.0, 2.0, True))
    d = jet.desc()
    assert (d.random.kind, d.random.cells_id, d.random.fraction) == (A.RND_CELLS, 3, 0.5)
    assert d.bfield.kind == A.B_HELICAL_CONICAL and d.bfield.in_plasma_frame == 0
    jet.bfield = J.PointsRandomVectorBField(b, 0.25, seed=9)
    d = jet.desc()
    assert (d.random.kind, d.random.seed, d.random.fraction) == (A.RND_POINTS, 9, 0.25)
    with pytest.raises(ValueError):
        J.PointsRandomVectorBField(J.RandomScalarBField(0.1, 1.0), 0.1)
