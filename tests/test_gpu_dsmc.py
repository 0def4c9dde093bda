"""DSMC on the device (PIC.perform!(::DirectSimulationMonteCarlo),
Chemistry/src/dsmc.jl:86-138) against the oracle: the carried remainder per
cell (deterministic: exact to FP64 rounding), momentum and energy
conservation of elastic collisions between equal weights (FP32 velocities),
the number of accepted collisions (statistically, against the oracle's own
random run), reproducibility, and the sets inside the step graph."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
from oracle import dsmc_oracle as do  # noqa: E402

pytestmark = pytest.mark.gpu

ME, MP = 9.1093837015e-31, 1.67262192e-27
N, D = 9, 0.05          # 8x8 cells of 5 cm
G = [3e6, 4e6, 5e6, 6e6]
S = [0.01, 0.1, 2.0, 0.01]  # the cross section of problem/05_dsmc.jl


def _state(seed, na=3000, nb=2000):
    r = np.random.default_rng(seed)
    L = (N - 1) * D
    # positions well inside their cells (no cell decided by rounding)
    def pos(n):
        c = r.integers(0, N - 1, (n, 2))
        return np.asfortranarray((c + r.uniform(0.05, 0.95, (n, 2))) * D)
    xa, xb = pos(na), pos(nb)
    va = np.asfortranarray(r.normal(0, 2.5e6, (na, 3)))
    vb = np.asfortranarray(r.normal(0, 3e3, (nb, 3)))
    assert xa.max() < L and xb.max() < L
    return xa, va, xb, vb


def _ctx(lib, xa, va, xb, vb, wa=1.0, wb=1.0):
    from iskra_gb300.device import Context
    ctx = Context(N, N, D, D, (0, 0, 0, 0))
    a = ctx.species_create(0.0, ME, wa, 2 * len(xa))
    b = ctx.species_create(0.0, 8 * MP, wb, 2 * len(xb))
    for s in (a, b):
        ctx.set_boundary(s, lib.BND_WRAP, lib.BND_WRAP)
    ctx.upload(a, xa, va, ids=np.arange(len(xa), dtype=np.uint32))
    ctx.upload(b, xb, vb, ids=np.arange(len(xb), dtype=np.uint32))
    k = ctx.dsmc_create(a, b, G, S)
    return ctx, a, b, k


def _vel(ctx, sid):
    x, v, ids = ctx.download(sid)
    o = np.argsort(ids)
    return x[o], v[o]


def test_dsmc_remainder_conservation_and_rate(lib):
    xa, va, xb, vb = _state(1)
    ctx, a, b, k = _ctx(lib, xa, va, xb, vb)
    xa, va = _vel(ctx, a)  # the device representation (FP32 velocities)
    xb, vb = _vel(ctx, b)
    dt = 2e-12
    rem = np.zeros(N * N)
    acc_gpu = acc_orc = 0
    va_o, vb_o = va.copy(), vb.copy()
    for step in range(3):
        ctx.dsmc_perform(k, dt, seed=9, step=step)
        rem_g, nu_g = ctx.dsmc_state(k)
        va_o, vb_o, rem, nu_o = do.perform(xa, va_o, xb, vb_o, ME, 8 * MP, 1.0, 1.0, G, S, (N, N, D, D), dt, rem,
                                           rng=np.random.default_rng(step))
        # the remainder depends only on the counts: equal to FP64 rounding
        assert np.allclose(rem_g.ravel(order="F"), rem, rtol=0, atol=1e-9)
        acc_gpu += int(nu_g.sum())
        acc_orc += int(nu_o.sum())
    assert acc_orc > 200
    assert abs(acc_gpu - acc_orc) < 6 * np.sqrt(acc_orc) + 10, (acc_gpu, acc_orc)
    _, va2 = _vel(ctx, a)
    _, vb2 = _vel(ctx, b)
    ma, mb = ME, 8 * MP
    p0 = ma * va.sum(0) + mb * vb.sum(0)
    p1 = ma * va2.sum(0) + mb * vb2.sum(0)
    scale = ma * np.abs(va).sum() + mb * np.abs(vb).sum()
    assert np.all(np.abs(p1 - p0) < 1e-5 * scale)
    e0 = ma * (va ** 2).sum() + mb * (vb ** 2).sum()
    e1 = ma * (va2 ** 2).sum() + mb * (vb2 ** 2).sum()
    assert np.isclose(e0, e1, rtol=1e-5)
    assert not np.array_equal(va, va2)  # collisions changed velocities
    ctx.close()


def test_dsmc_is_reproducible(lib):
    xa, va, xb, vb = _state(2)
    outs = []
    for _ in range(2):
        ctx, a, b, k = _ctx(lib, xa, va, xb, vb)
        ctx.dsmc_perform(k, 2e-12, seed=4, step=1)
        outs.append((_vel(ctx, a)[1], _vel(ctx, b)[1]))
        ctx.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_dsmc_in_step_graph(lib):
    """iskra_step performs the DSMC set every step (after the MCC sets,
    before the push)."""
    EPS0 = 8.8541878128e-12
    xa, va, xb, vb = _state(3)
    ctx, a, b, k = _ctx(lib, xa, va, xb, vb)
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    left = np.zeros((N, N), bool)
    left[0, :] = True
    ctx.apply_dirichlet(left, 0.0)
    e0 = ME * (_vel(ctx, a)[1] ** 2).sum() + 8 * MP * (_vel(ctx, b)[1] ** 2).sum()
    ctx.step(2e-12, 4, seed=2, rtol=1e-8)
    ctx.sync()
    _, nu = ctx.dsmc_state(k)
    assert nu.sum() > 0
    e1 = ME * (_vel(ctx, a)[1] ** 2).sum() + 8 * MP * (_vel(ctx, b)[1] ** 2).sum()
    assert np.isclose(e0, e1, rtol=1e-4)  # uncharged species: no field work
    ctx.close()


@pytest.mark.parametrize("same", [False, True])
def test_dsmc_crowded_cells(lib, same):
    """Cells with more lists than shared memory stages (above 512 particles)
    take the global-memory path: remainder against the oracle, accepted
    collisions against the oracle's own random run, momentum and energy
    conserved, and the result reproducible (independent of the order in
    which the cell lists were scattered)."""
    from iskra_gb300.device import Context
    n, d, dt = 3, 0.05, 5e-13  # 2x2 cells
    r = np.random.default_rng(11)
    na, nb = 3000, 2400

    def pos(m):
        c = r.integers(0, n - 1, (m, 2))
        return np.asfortranarray((c + r.uniform(0.05, 0.95, (m, 2))) * d)

    xa, xb = pos(na), pos(nb)
    va = np.asfortranarray(r.normal(0, 2.5e6, (na, 3)))
    vb = np.asfortranarray(r.normal(0, 3e3, (nb, 3)))
    ma, mb = ME, (ME if same else 8 * MP)

    def make():
        ctx = Context(n, n, d, d, (0, 0, 0, 0))
        a = ctx.species_create(0.0, ma, 1.0, 2 * na)
        ctx.set_boundary(a, lib.BND_WRAP, lib.BND_WRAP)
        ctx.upload(a, xa, va, ids=np.arange(na, dtype=np.uint32))
        b = a
        if not same:
            b = ctx.species_create(0.0, mb, 1.0, 2 * nb)
            ctx.set_boundary(b, lib.BND_WRAP, lib.BND_WRAP)
            ctx.upload(b, xb, vb, ids=np.arange(nb, dtype=np.uint32))
        return ctx, a, b, ctx.dsmc_create(a, b, G, S)

    ctx, a, b, k = make()
    x0a, v0a = _vel(ctx, a)
    x0b, v0b = _vel(ctx, b)
    counts = np.bincount((x0a[:, 0] // d).astype(int) + 2 * (x0a[:, 1] // d).astype(int), minlength=4)
    assert counts.min() > 512
    rem = np.zeros(n * n)
    acc_gpu = acc_orc = 0
    va_o, vb_o = v0a.copy(), v0b.copy()
    for step in range(2):
        ctx.dsmc_perform(k, dt, seed=7, step=step)
        rem_g, nu_g = ctx.dsmc_state(k)
        va_o, vb_o, rem, nu_o = do.perform(x0a, va_o, x0b, vb_o, ma, mb, 1.0, 1.0, G, S, (n, n, d, d), dt, rem,
                                           same=same, rng=np.random.default_rng(100 + step))
        assert np.allclose(rem_g.ravel(order="F"), rem, rtol=0, atol=1e-9)
        acc_gpu += int(nu_g.sum())
        acc_orc += int(nu_o.sum())
    assert acc_orc > 200
    assert abs(acc_gpu - acc_orc) < 6 * np.sqrt(acc_orc) + 10, (acc_gpu, acc_orc)
    _, v1a = _vel(ctx, a)
    _, v1b = _vel(ctx, b)
    ctx.close()
    if same:
        p0, p1 = ma * v0a.sum(0), ma * v1a.sum(0)
        e0, e1 = ma * (v0a ** 2).sum(), ma * (v1a ** 2).sum()
        scale = ma * np.abs(v0a).sum()
    else:
        p0, p1 = ma * v0a.sum(0) + mb * v0b.sum(0), ma * v1a.sum(0) + mb * v1b.sum(0)
        e0, e1 = ma * (v0a ** 2).sum() + mb * (v0b ** 2).sum(), ma * (v1a ** 2).sum() + mb * (v1b ** 2).sum()
        scale = ma * np.abs(v0a).sum() + mb * np.abs(v0b).sum()
    assert np.all(np.abs(p1 - p0) < 1e-5 * scale)
    assert np.isclose(e0, e1, rtol=1e-5)
    assert not np.array_equal(v0a, v1a)
    # the same perform! again on a fresh context: bit-identical
    ctx, a, b, k = make()
    ctx.dsmc_perform(k, dt, seed=7, step=0)
    ctx.dsmc_perform(k, dt, seed=7, step=1)
    assert np.array_equal(_vel(ctx, a)[1], v1a)
    if not same:
        assert np.array_equal(_vel(ctx, b)[1], v1b)
    ctx.close()
