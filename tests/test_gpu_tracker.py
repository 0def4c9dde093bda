"""Surface tracker in the GPU push (track! + check! + hit!, pic/surfaces/*.jl,
circuit_coupling.jl:45-63) against the FP64 oracle: which particles each
surface absorbs (exact, by id), the positions and velocities after
reflections, the hit counts and the σ credit of a floating electrode.
Particles whose walk has a comparison closer than 1e-3 (of a cell or of the
step) are left out, so FP32 arithmetic on the device cannot decide them
differently from the oracle."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
from oracle import tracker_oracle as to  # noqa: E402

pytestmark = pytest.mark.gpu

QE, ME, EPS0 = 1.602176634e-19, 9.1093837015e-31, 8.8541878128e-12


def _setup(lib, n, d):
    from iskra_gb300.device import Context
    ctx = Context(n, n, d, d, (0, 0, 0, 0))
    ctx.poisson_create(EPS0)
    left = np.zeros((n, n), bool)
    left[0, :] = True
    ctx.apply_dirichlet(left, 0.0)
    return ctx


def _surfaces(n):
    block = np.zeros((n, n), bool)
    block[10:15, 10:15] = True           # reflective 5x5-node block
    fixed = np.zeros((n, n), bool)
    fixed[24, 4:28] = True               # fixed electrode: a node column
    floating = np.zeros((n, n), bool)
    floating[4:20, 26] = True            # floating electrode: a node row
    periodic = np.zeros((n, n), bool)
    periodic[5, 2:9] = True              # a transparent (periodic) segment
    return block, fixed, floating, periodic


@pytest.mark.parametrize("default", ["absorb", "reflect"])
def test_tracker_matches_oracle(lib, default):
    n, d, dt = 33, 1e-3, 1e-10
    w0, npart = 1e5, 60000
    ctx = _setup(lib, n, d)
    dkind = lib.SURF_ABSORB if default == "absorb" else lib.SURF_REFLECT
    block, fixed, floating, periodic = _surfaces(n)
    dof = ctx.add_dof()
    ctx.apply_neumann(floating, dof)
    ctx.set_sigma(dof, 1e-9)
    area = float(d * np.count_nonzero(floating[:-1, :] & floating[1:, :])
                 + d * np.count_nonzero(floating[:, :-1] & floating[:, 1:]))
    ctx.tracker_create(dkind)
    f_block = ctx.tracker_add_surface(block, lib.SURF_REFLECT)
    f_fixed = ctx.tracker_add_surface(fixed, lib.SURF_FIXED)
    f_float = ctx.tracker_add_surface(floating, lib.SURF_FLOATING, dof, area)
    f_per = ctx.tracker_add_surface(periodic, lib.SURF_PERIODIC)

    tr = to.Tracker(n, n, to.ABSORB if default == "absorb" else to.REFLECT)
    assert tr.add(block, to.REFLECT) == f_block
    assert tr.add(fixed, to.FIXED) == f_fixed
    assert tr.add(floating, to.FLOATING) == f_float
    assert tr.add(periodic, to.PERIODIC) == f_per

    sid = ctx.species_create(-QE, ME, w0, 2 * npart)
    ctx.set_boundary(sid, lib.BND_DISCARD, lib.BND_DISCARD)
    r = np.random.default_rng(11)
    L = (n - 1) * d
    vmax = 0.9 * d / dt
    x = np.asfortranarray(r.uniform(0.02 * L, 0.98 * L, (npart, 2)))
    v = np.asfortranarray(np.column_stack([r.uniform(-vmax, vmax, (npart, 2)), r.normal(0, 1e5, npart)]))
    # the device representation of the inputs (cell + offset on the 2^-24 grid, FP32 velocity)
    ctx.upload(sid, x, v)
    x0, v0, _ = ctx.download(sid)
    keep = to.decision_margin(tr, x0, v0, dt, d, d) > 1e-3
    x0, v0 = np.asfortranarray(x0[keep]), np.asfortranarray(v0[keep])
    ids = np.arange(len(x0), dtype=np.uint32)
    ctx.upload(sid, x0, v0, ids=ids)
    x0b, v0b, id0 = ctx.download(sid)  # (in tile order: the upload sorts)
    o = np.argsort(id0)
    assert np.array_equal(id0[o], ids)
    assert np.array_equal(x0b[o], x0) and np.array_equal(v0b[o], v0)
    ctx.upload_E(np.zeros((n, n, 3)))
    sig0 = ctx.get_sigma(dof)

    ctx.advance(sid, dt)
    x1, v1, id1 = ctx.download(sid)

    xo, vo, ab, hits, dsig = to.advance_tracked(tr, x0, v0, dt, d, d, qw=-QE * w0, areas={f_float: area})
    # after_push discard! of what left the grid untracked (none: walls are surfaces)
    inside = (xo[:, 0] >= 0) & (xo[:, 0] < L) & (xo[:, 1] >= 0) & (xo[:, 1] < L)
    survive = ~ab & inside
    assert set(id1.tolist()) == set(ids[survive].tolist())
    order = np.argsort(id1)
    x1, v1 = x1[order], v1[order]
    assert np.allclose(x1, xo[survive], rtol=0, atol=1e-9)
    assert np.allclose(v1[:, :2], vo[survive, :2], rtol=1e-6, atol=0)
    for f in range(len(tr.kinds)):
        assert ctx.tracker_hits(f, sid) == hits[f], f
    assert hits[f_block] == 0 and hits[f_per] == 0
    assert hits[f_fixed] > 0 and hits[f_float] > 0
    if default == "absorb":
        assert hits[0] > 0
    # reflections happened and were reproduced
    flipped = np.sign(vo[survive, 0]) != np.sign(v0[survive, 0])
    assert flipped.sum() > 10
    assert np.isclose(ctx.get_sigma(dof) - sig0, dsig[f_float], rtol=1e-12, atol=0)
    ctx.close()


def test_step_graph_credits_floating_electrode(lib):
    """Inside iskra_step (one captured graph) the floating electrode's σ
    gains q w / area per absorbed particle before the field solve."""
    n, d, dt = 33, 1e-3, 1e-10
    w0, npart = 1e4, 40000
    ctx = _setup(lib, n, d)
    _, _, floating, _ = _surfaces(n)
    dof = ctx.add_dof()
    ctx.apply_neumann(floating, dof)
    area = float(d * np.count_nonzero(floating[:-1, :] & floating[1:, :]))
    ctx.tracker_create(lib.SURF_ABSORB)
    f = ctx.tracker_add_surface(floating, lib.SURF_FLOATING, dof, area)
    sid = ctx.species_create(-QE, ME, w0, npart)
    ctx.set_boundary(sid, lib.BND_DISCARD, lib.BND_DISCARD)
    r = np.random.default_rng(5)
    L = (n - 1) * d
    x = np.asfortranarray(r.uniform(0.05 * L, 0.95 * L, (npart, 2)))
    v = np.asfortranarray(r.normal(0, 2e6, (npart, 3)))
    ctx.upload(sid, x, v)
    s0 = ctx.get_sigma(dof)
    ctx.step(dt, 5, seed=1, rtol=1e-8)
    ctx.sync()
    h = ctx.tracker_hits(f, sid)
    assert h > 0
    assert np.isclose(ctx.get_sigma(dof) - s0, -QE * w0 * h / area, rtol=1e-12, atol=0)
    ctx.close()
