"""The plain-method 1D configuration (two counter-streaming electron beams on
a neutralising ion background, periodic in x, problem/10_two_streams.jl, at
the configuration's L = 0.1 m, 128 nodes, ±1e6 m/s, 1e11 m^-3 per beam):
GPU (iskra_step, one CUDA graph per step) against the oracle from the same
initial particles.  At these parameters every mode that fits the domain has
k v0 >= 2π/L x 1e6 m/s = 6.3e7 1/s, above the beams' instability bound
√2 ω_p = 2.5e7 1/s, so the field energy stays at the seeded noise level; the
two runs are compared through their field-energy histories sampled every 10
steps, which follow the particles' positions step by step.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QE = 1.602176634e-19
ME = 9.1093837015e-31
EPS0 = 8.8541878128e-12

L, NX, NY = 0.1, 128, 2
DX = L / (NX - 1)            # wrap period (n-1)Δx = L
NB, N0 = 20000, 1e11         # macroparticles and density per beam
DT, STEPS, EVERY = 2e-9, 2000, 10


def field_energy(E):
    return 0.5 * EPS0 * np.sum(E[:, :, 0] ** 2 + E[:, :, 1] ** 2) * DX * DX


def initial_state():
    rng = np.random.default_rng(1)
    x = np.column_stack([rng.uniform(0, L, 2 * NB), rng.uniform(0, DX, 2 * NB)])
    v = np.zeros((2 * NB, 3))
    v[:NB, 0] = 1e6 + 1e4 * rng.standard_normal(NB)
    v[NB:, 0] = -1e6 + 1e4 * rng.standard_normal(NB)
    return np.asfortranarray(x), np.asfortranarray(v)


def test_two_stream_growth_matches_oracle(orc, lib):
    from iskra_gb300.device import Context
    w = N0 * L * DX / NB
    x, v = initial_state()
    bg = np.full((NX, NY), QE * 2 * N0)

    ctx = Context(NX, NY, DX, DX, (1, 1, 1, 1))
    se = ctx.species_create(-QE, ME, w, 2 * NB)
    ctx.set_boundary(se, lib.BND_WRAP, lib.BND_WRAP)
    ctx.upload(se, x, v)
    ctx.set_background(bg)
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    ctx.apply_periodic(2)
    Wg = []
    for k in range(STEPS // EVERY):
        ctx.step(DT, EVERY, seed=0, rtol=1e-10)
        Wg.append(field_energy(ctx.field(lib.FIELD_E)))
    ctx.close()

    po = orc.PicOracle(NX, NY, DX, DX, EPS0, bcs=(1, 1, 1, 1))
    po.add_species(-QE, ME, w, 2 * NB, x, v, bnd=(1, 1))
    po.background = bg
    po.ps.apply_periodic(1)
    po.ps.apply_periodic(2)
    Wo = []
    for s in range(STEPS):
        po.step(DT, s)
        if (s + 1) % EVERY == 0:
            Wo.append(field_energy(po.E))

    Wg, Wo = np.array(Wg), np.array(Wo)
    rel = np.abs(Wg - Wo) / Wo
    # the same field energy at every checkpoint of the first 200 steps, and a
    # closely matching history and level over the whole run
    assert rel[:20].max() < 1e-2, rel[:20]
    assert np.median(rel) < 0.05, np.round(rel, 4)
    assert abs(Wg.mean() / Wo.mean() - 1) < 0.05, (Wg.mean(), Wo.mean())
