"""CPU oracle of the particle sources -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` imports this module, as the checker of the device sampler
(``iskra_gb300/csrc/source.cu``).  Restates sample!(::MaxwellianSource,
species, Δt) (ParticleInCell/src/pic/sources.jl:24-34) with numpy's
generator: n = min(free slots, floor(rate Δt)), px = rand(n, D) wx + dx,
pv = randn(n, V) wv + dv.  Julia's random stream cannot be reproduced, so the
device sample is compared with this one statistically (parity unpinned).
"""
from __future__ import annotations

import numpy as np


def count(rate, dt, np_live, capacity):
    """n of sources.jl:30 (min of the free slots and floor(rate Δt))."""
    return int(max(0, min(capacity - np_live, int(np.floor(rate * dt)))))


def sample(rate, dt, wx, wv, dx=None, dv=None, np_live=0, capacity=None, rng=None):
    """(x (n, 2), v (n, 3)) of one sample!."""
    rng = np.random.default_rng(0) if rng is None else rng
    wx, wv = np.asarray(wx, float).ravel(), np.asarray(wv, float).ravel()
    dx = np.zeros(2) if dx is None else np.asarray(dx, float).ravel()
    dv = np.zeros(3) if dv is None else np.asarray(dv, float).ravel()
    cap = np_live + int(np.floor(rate * dt)) if capacity is None else capacity
    n = count(rate, dt, np_live, cap)
    x = rng.random((n, 2)) * wx + dx
    v = rng.standard_normal((n, 3)) * wv + dv
    return x, v


def moments(wx, wv, dx=None, dv=None):
    """Exact means and variances of the sampled x (uniform) and v (normal)."""
    wx, wv = np.asarray(wx, float).ravel(), np.asarray(wv, float).ravel()
    dx = np.zeros(2) if dx is None else np.asarray(dx, float).ravel()
    dv = np.zeros(3) if dv is None else np.asarray(dv, float).ravel()
    return dx + wx / 2, wx ** 2 / 12, dv, wv ** 2
