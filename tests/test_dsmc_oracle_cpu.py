"""The DSMC oracle (dsmc.jl:86-138) against its definition: σgmax, the pairs
tried per cell with the carried remainder, conservation in elastic
collisions of equal weights."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
from oracle import dsmc_oracle as do  # noqa: E402


def test_sgmax_is_max_sigma_times_its_g():
    assert do.sgmax([3e6, 4e6, 5e6, 6e6], [0.01, 0.1, 2.0, 0.01]) == 2.0 * 5e6


def test_pairs_and_remaining():
    n, rem = do.pairs_and_remaining([10, 1, 10], [5, 5, 1], 1.0, 1.0, 0.1, 0.1, 1e-3, 2.0, False, np.array([0.5, 0.3, 0.2]))
    # cell 0: na = 10/0.01 = 1000, Nc = 1000*5*1e-3*2 / 2 * 2 + 0.5 = 10.5
    assert n[0] == 10 and np.isclose(rem[0], 0.5)
    assert n[1] == 0 and rem[1] == 0.3 and n[2] == 0 and rem[2] == 0.2


def test_elastic_collisions_conserve_momentum_and_energy():
    r = np.random.default_rng(4)
    nx = ny = 4
    dx = dy = 0.1
    xa = r.uniform(0.01, 0.39, (400, 2))
    xb = r.uniform(0.01, 0.39, (300, 2))
    va = r.normal(0, 4e6, (400, 3))
    vb = r.normal(0, 1e5, (300, 3))
    ma, mb = 1.0, 3.0
    va2, vb2, rem, nu = do.perform(xa, va, xb, vb, ma, mb, 1.0, 1.0, [1e6, 5e6], [1e-3, 1e-3],
                                   (nx, ny, dx, dy), 1e-7, np.zeros(nx * ny), rng=np.random.default_rng(1))
    assert nu.sum() > 20
    p0 = ma * va.sum(0) + mb * vb.sum(0)
    p1 = ma * va2.sum(0) + mb * vb2.sum(0)
    assert np.allclose(p0, p1, rtol=1e-9, atol=1e-9 * np.abs(ma * va).sum())
    e0 = ma * (va ** 2).sum() + mb * (vb ** 2).sum()
    e1 = ma * (va2 ** 2).sum() + mb * (vb2 ** 2).sum()
    assert np.isclose(e0, e1, rtol=1e-12)


def _nc_literal(Na, Nb, Wa, Wb, dx, dy, dt, sgm, same, rem):
    """dsmc.jl:94-117 transcribed line by line for one cell."""
    if Wa > Wb:
        Pab, Pba = Wb / Wa, 1.0
    else:
        Pab, Pba = 1.0, Wa / Wb
    if Na < 2 or Nb < 2:
        return 0, rem
    na = Na * Wa / (dx * dy)
    Nc = na * Nb * dt * sgm
    Nc /= Pab + (Wb / Wa) * Pba
    if not same:
        Nc *= 2
    Nc += rem
    return int(np.floor(Nc)), Nc - np.floor(Nc)


def test_pairs_and_remaining_match_the_literal_loop():
    r = np.random.default_rng(7)
    for same in (False, True):
        for Wa, Wb in ((1.0, 1.0), (2.0, 0.5), (0.3, 3.0)):
            Na = r.integers(0, 40, 200)
            Nb = Na if same else r.integers(0, 40, 200)
            rem = r.random(200)
            n, new = do.pairs_and_remaining(Na, Nb, Wa, Wb, 0.05, 0.02, 3e-9, 7e6, same, rem)
            for k in range(200):
                nk, rk = _nc_literal(int(Na[k]), int(Nb[k]), Wa, Wb, 0.05, 0.02, 3e-9, 7e6, same, rem[k])
                assert n[k] == nk and new[k] == rk
