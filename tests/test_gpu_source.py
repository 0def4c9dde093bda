"""Particle sources on the device (sample!, pic/sources.jl:24-34) against the
oracle: the count (exact, capped by the capacity), identifiers continuing the
species' counter, the distributions (means and variances within 5 standard
errors of the exact values, two-sample Kolmogorov-Smirnov test against the
oracle's sample), reproducibility, and sampling inside the step graph."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
from oracle import source_oracle as so  # noqa: E402

pytestmark = pytest.mark.gpu

QE, ME, EPS0 = 1.602176634e-19, 9.1093837015e-31, 8.8541878128e-12
N, D = 65, 1e-3
L = (N - 1) * D
WX, DX = [0.5 * L, 0.25 * L], [0.25 * L, 0.5 * L]
WV, DV = [1e5, 2e5, 3e5], [1e4, 0.0, -1e4]


def _ctx(lib, cap):
    from iskra_gb300.device import Context
    ctx = Context(N, N, D, D, (0, 0, 0, 0))
    sid = ctx.species_create(-QE, ME, 1.0, cap)
    ctx.set_boundary(sid, lib.BND_WRAP, lib.BND_WRAP)
    return ctx, sid


def test_source_count_capacity_and_ids(lib):
    ctx, sid = _ctx(lib, 100000)
    r = np.random.default_rng(2)
    x = np.asfortranarray(r.uniform(0, L, (10000, 2)))
    v = np.asfortranarray(r.normal(0, 1e5, (10000, 3)))
    ctx.upload(sid, x, v)
    src = ctx.source_create(sid, 5e13, WX, WV, DX, DV)  # 50000 per 1 ns
    ctx.source_sample(src, 1e-9, seed=7)
    assert ctx.count(sid) == 60000
    ctx.source_sample(src, 1e-9, seed=7)  # 40000 free slots
    assert ctx.count(sid) == so.count(5e13, 1e-9, 60000, 100000) + 60000 == 100000
    ctx.source_sample(src, 1e-9, seed=7)  # full: nothing added
    assert ctx.count(sid) == 100000
    _, _, ids = ctx.download(sid)
    assert len(np.unique(ids)) == 100000
    assert set(range(10001, 100001)).issubset(set(ids.tolist()))
    ctx.close()


def test_source_distribution_matches_oracle(lib):
    from scipy import stats
    ctx, sid = _ctx(lib, 400000)
    src = ctx.source_create(sid, 4e14, WX, WV, DX, DV)
    ctx.source_sample(src, 1e-9, seed=11)
    x, v, _ = ctx.download(sid)
    n = len(x)
    assert n == 400000
    mx, vx, mv, vv = so.moments(WX, WV, DX, DV)
    assert np.all(np.abs(x.mean(0) - mx) < 5 * np.sqrt(vx / n))
    assert np.all(np.abs(v.mean(0) - mv) < 5 * np.sqrt(vv / n))
    assert np.allclose(x.var(0), vx, rtol=0.02) and np.allclose(v.var(0), vv, rtol=0.02)
    assert np.all(x >= np.asarray(DX) - 1e-12) and np.all(x < np.asarray(DX) + WX)
    xo, vo = so.sample(4e14, 1e-9, WX, WV, DX, DV, rng=np.random.default_rng(3))
    for a in range(2):
        assert stats.ks_2samp(x[:, a], xo[:, a]).pvalue > 1e-4, a
    for a in range(3):
        assert stats.ks_2samp(v[:, a], vo[:, a]).pvalue > 1e-4, a
    ctx.close()


def test_source_is_reproducible(lib):
    outs = []
    for _ in range(2):
        ctx, sid = _ctx(lib, 20000)
        src = ctx.source_create(sid, 1e13, WX, WV, DX, DV)
        ctx.source_sample(src, 1e-9, seed=5)
        ctx.source_sample(src, 1e-9, seed=5)
        x, v, ids = ctx.download(sid)
        o = np.argsort(ids)
        outs.append((x[o], v[o]))
        ctx.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    # the second call of the same seed draws new values
    assert not np.array_equal(outs[0][0][:10000], outs[0][0][10000:])


def test_source_every_step_in_graph(lib):
    """Sampled at the start of each iskra_step (ParticleInCell.jl:104-106),
    inside the captured step graph: the count grows by floor(rate Δt) per
    step (walls wrap, nothing is lost) and the samples of different steps
    differ."""
    ctx, sid = _ctx(lib, 200000)
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    left = np.zeros((N, N), bool)
    left[0, :] = True
    right = np.zeros((N, N), bool)
    right[-1, :] = True
    ctx.apply_dirichlet(left, 0.0)
    ctx.apply_dirichlet(right, 0.0)
    src = ctx.source_create(sid, 2e12, WX, [1e3, 1e3, 1e3], DX, None)  # 200 per 1e-10 s
    ctx.source_every_step(src, True)
    ctx.step(1e-10, 10, seed=3, rtol=1e-8)
    ctx.sync()
    assert ctx.count(sid) == 2000
    ctx.step(1e-10, 15, seed=3, rtol=1e-8)
    ctx.sync()
    assert ctx.count(sid) == 5000
    x, v, ids = ctx.download(sid)
    assert len(np.unique(ids)) == 5000
    ctx.close()
