"""The surface-tracker oracle against trajectories worked out by hand from
ParticleInCell/src/pic/surfaces/*.jl (the reference has no tracker tests or
fixtures of its own)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
from oracle import tracker_oracle as to  # noqa: E402


def _one(tr, x, v, dt=1.0, d=1.0, **kw):
    return to.advance_tracked(tr, np.array([x], float), np.array([v + [0.0]], float), dt, d, d, **kw)


def test_default_walls_absorb():
    tr = to.Tracker(10, 10)
    # cell (9, 5) borders the x-high wall (x = 9): crossing it absorbs
    x, v, ab, hits, _ = _one(tr, [8.5, 4.5], [1.0, 0.0])
    assert ab[0] and hits[0] == 1
    # staying inside the boundary cell: untouched
    x, v, ab, hits, _ = _one(tr, [8.2, 4.5], [0.5, 0.0])
    assert not ab[0] and hits[0] == 0 and np.allclose(x[0], [8.7, 4.5])


def test_reflective_wall_mirrors_the_rest_of_the_step():
    tr = to.Tracker(10, 10)
    nodes = np.zeros((10, 10), bool)
    nodes[4, :] = True  # 1-based node column 5: the edge x = 4 between cells 4 and 5
    tr.add(nodes, to.REFLECT)
    x, v, ab, hits, _ = _one(tr, [3.5, 4.5], [1.0, 0.25])
    # crosses x = 4 after 0.5, comes back 0.5: x = 3.5; y moves the full step
    assert not ab[0]
    assert np.allclose(x[0], [3.5, 4.75]) and np.allclose(v[0, :2], [-1.0, 0.25])
    # from the other side as well
    x, v, ab, hits, _ = _one(tr, [4.25, 4.5], [-0.5, 0.0])
    assert np.allclose(x[0], [4.25, 4.5]) and np.allclose(v[0, :2], [0.5, 0.0])


def test_periodic_surface_is_transparent():
    tr = to.Tracker(10, 10)
    nodes = np.zeros((10, 10), bool)
    nodes[4, :] = True
    tr.add(nodes, to.PERIODIC)
    x, v, ab, hits, _ = _one(tr, [3.5, 4.5], [1.0, 0.0])
    assert not ab[0] and np.allclose(x[0], [4.5, 4.5]) and hits.sum() == 0


def test_floating_electrode_counts_charge():
    tr = to.Tracker(10, 10)
    nodes = np.zeros((10, 10), bool)
    nodes[2:5, 2:5] = True  # a 3x3-node block: cells (3,3),(4,3),(3,4),(4,4) 1-based
    f = tr.add(nodes, to.FLOATING)
    # from cell (2, 4) (x in [1, 2)) moving +x into the block at x = 2
    x, v, ab, hits, dsig = _one(tr, [1.5, 3.5], [1.0, 0.0], qw=-2.0, areas={f: 4.0})
    assert ab[0] and hits[f] == 1 and np.isclose(dsig[f], -0.5)
    # the block's edges are surfaces from inside too
    x, v, ab, hits, dsig = _one(tr, [3.5, 3.5], [0.0, -2.0], qw=-2.0, areas={f: 4.0})
    assert ab[0] and hits[f] == 1


def test_later_surfaces_replace_earlier_ones():
    tr = to.Tracker(10, 10)
    nodes = np.zeros((10, 10), bool)
    nodes[4, :] = True
    tr.add(nodes, to.ABSORB)
    tr.add(nodes, to.REFLECT)
    x, v, ab, hits, _ = _one(tr, [3.5, 4.5], [1.0, 0.0])
    assert not ab[0] and np.allclose(x[0], [3.5, 4.5])


def test_untracked_cells_are_not_walked():
    tr = to.Tracker(10, 10)
    assert (5, 5) not in tr.tracked_cells()
    x, v, ab, hits, _ = _one(tr, [4.5, 4.5], [0.3, 0.2])
    assert not ab[0] and np.allclose(x[0], [4.8, 4.7])


def test_diagonal_crossing_walks_two_edges():
    tr = to.Tracker(10, 10)
    nodes = np.zeros((10, 10), bool)
    nodes[:, 4] = True  # the edge y = 4 (1-based node row 5)
    tr.add(nodes, to.REFLECT)
    # from (3.8, 3.7): x edge at t = 0.4 (no surface), then y edge at t = 0.6
    x, v, ab, hits, _ = _one(tr, [3.8, 3.7], [0.5, 0.5])
    assert not ab[0]
    assert np.allclose(x[0], [4.3, 4.0 - 0.2]) and np.allclose(v[0, :2], [0.5, -0.5])


def test_reflection_is_the_mirror_image_and_walls_absorb_escapes():
    """Known answers from geometry, independent of the walk: with a
    reflective wall along x = 4 (cell units) and absorbing domain walls, a
    straight path of less than a cell either stays free, ends at its mirror
    image about x = 4 with v_x flipped, or leaves the domain and is absorbed."""
    tr = to.Tracker(10, 10)
    nodes = np.zeros((10, 10), bool)
    nodes[4, :] = True
    f = tr.add(nodes, to.REFLECT)
    r = np.random.default_rng(3)
    n = 3000
    x0 = r.uniform(0.02, 8.98, (n, 2))
    v = np.column_stack([r.uniform(-0.95, 0.95, (n, 2)), np.zeros(n)])
    free = x0 + v[:, :2]
    # keep paths that cross at most one of {x = 4, the walls} and stay away from corners/edges of the decision
    cross_wall = (np.sign(x0[:, 0] - 4) != np.sign(free[:, 0] - 4))
    leaves = (free < 0).any(1) | (free > 9).any(1)
    near = (np.abs(free[:, 0] - 4) < 1e-6) | (np.abs(x0[:, 0] - 4) < 1e-6)
    keep = ~near & ~(cross_wall & leaves)
    x, vo, ab, hits, _ = to.advance_tracked(tr, x0[keep], v[keep], 1.0, 1.0, 1.0)
    cw, lv, fr, v0 = cross_wall[keep], leaves[keep], free[keep], v[keep]
    # escapes are absorbed by the default walls (surface 0), nothing else is
    assert np.array_equal(ab, lv) and hits[0] == lv.sum() and hits[f] == 0
    ok = ~lv
    mirror = fr.copy()
    mirror[cw, 0] = 8.0 - fr[cw, 0]
    assert np.allclose(x[ok], mirror[ok], atol=1e-12)
    flip = np.where(cw, -1.0, 1.0)
    assert np.allclose(vo[ok, 0], (flip * v0[:, 0])[ok]) and np.allclose(vo[ok, 1], v0[ok, 1])
