"""The source oracle (sample!, pic/sources.jl:24-34) against its definition."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
from oracle import source_oracle as so  # noqa: E402


def test_count_is_capped_by_capacity():
    assert so.count(1e12, 1e-9, 0, 10000) == 1000
    assert so.count(1e12, 1e-9, 9500, 10000) == 500
    assert so.count(1e12, 1e-9, 10000, 10000) == 0
    assert so.count(0.5, 1.0, 0, 10) == 0  # floor(rate Δt)


def test_sample_moments():
    wx, dx = [2.0, 0.5], [1.0, -1.0]
    wv, dv = [3.0, 1.0, 0.25], [0.0, 5.0, -2.0]
    x, v = so.sample(2e5, 1.0, wx, wv, dx, dv, rng=np.random.default_rng(1))
    assert x.shape == (200000, 2) and v.shape == (200000, 3)
    mx, vx, mv, vv = so.moments(wx, wv, dx, dv)
    n = len(x)
    assert np.all(np.abs(x.mean(0) - mx) < 5 * np.sqrt(vx / n))
    assert np.all(np.abs(v.mean(0) - mv) < 5 * np.sqrt(vv / n))
    assert np.allclose(x.var(0), vx, rtol=0.02) and np.allclose(v.var(0), vv, rtol=0.02)
    assert np.all(x >= dx) and np.all(x < np.asarray(dx) + wx)
