"""The 2D discharge at full configuration size (1024 x 1024 nodes, 32 M
electrons + 32 M Ar+ ions, the discharge cross sections and gas, a driven
electrode at x = 0, a grounded one at x = max, y periodic) stepped through
iskra_step, checked by size-independent properties:

* particle bookkeeping: every ionisation child is one electron and one ion;
* the deposit conserves charge: Σ ρ V over the nodes equals Σ q w over the
  live particles (integer deposit; cell volumes halved on the electrode
  columns as cell_volume does);
* the Poisson solve met its tolerance, and E = -∇ϕ of the downloaded ϕ;
* MCC ran: collisions of every electron process were accepted.
"""
import numpy as np
import pytest

from test_gpu_discharge import EPS0, KB, M_AR, ME, QE, argon_tables

pytestmark = pytest.mark.gpu

NX = NY = 1024
GAP = 0.025
DX = GAP / (NX - 1)
NP = 32 * 1024 * 1024
DT = 7.4e-11
STEPS = 20


def test_full_size_discharge_properties(orc, lib):
    from iskra_gb300.device import Context
    rng = np.random.default_rng(5)
    w = 1e15 * GAP * GAP / NP
    ctx = Context(NX, NY, DX, DX, (0, 0, 1, 1))
    se = ctx.species_create(-QE, ME, w, NP + NP // 4)
    si = ctx.species_create(QE, M_AR, w, NP + NP // 4)
    for s in (se, si):
        ctx.set_boundary(s, lib.BND_DISCARD, lib.BND_WRAP)
    for s, T, m in ((se, 4.0, ME), (si, 0.03, M_AR)):
        x = np.empty((NP, 2), order="F")
        x[:, 0] = rng.uniform(0, GAP, NP)
        x[:, 1] = rng.uniform(0, GAP, NP)
        v = np.asfortranarray(rng.standard_normal((NP, 3)) * np.sqrt(2 * T * QE / m))
        ctx.upload(s, x, v)
        del x, v
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    left = np.zeros((NX, NY), bool)
    left[0, :] = True
    right = np.zeros((NX, NY), bool)
    right[-1, :] = True
    ctx.apply_dirichlet(left, 0.0)
    ctx.apply_dirichlet(right, 0.0)
    ctx.drive_dirichlet(left, 300.0, 13.56e6)
    assert ctx.set_method(0) == 0
    eps, el, ex, iz, cx = argon_tables()
    gas_n = np.full((NX, NY), 3.0 / (KB * 300.0))
    me_, _ = ctx.mcc_create(se, [(lib.MCC_ELASTIC_ISOTROPIC, 0.0, eps, el), (lib.MCC_EXCITATION, 11.5, eps, ex),
                                 (lib.MCC_IONIZATION, 15.76, eps, iz)], M_AR, 300.0, gas_n, product=si)
    mi_, _ = ctx.mcc_create(si, [(lib.MCC_ELASTIC_BACKWARD, 0.0, eps, cx)], M_AR, 300.0, gas_n)
    ctx.step(DT, STEPS, seed=7, rtol=1e-8)
    ctx.sync()
    it, relres = ctx.solve_info()
    assert relres <= 1e-8

    counts_e = ctx.mcc_counts(me_, 3)
    counts_i = ctx.mcc_counts(mi_, 1)
    assert all(c > 0 for c in counts_e) and counts_i[0] > 0
    n_e, n_i = ctx.count(se), ctx.count(si)
    ab_e, ab_i = ctx.absorbed(se), ctx.absorbed(si)
    # each ionising electron (at most one child per particle and step) adds
    # one electron and one ion (equal weights); accepted ionisation events
    # include those without the threshold energy
    created_e = n_e - (NP - sum(ab_e))
    created_i = n_i - (NP - sum(ab_i))
    assert created_e == created_i and 0 < created_e <= counts_e[2], (created_e, created_i, counts_e)

    rho = ctx.field(lib.FIELD_RHO)
    V = np.full((NX, NY), DX * DX)
    V[0, :] *= 0.5
    V[-1, :] *= 0.5
    total = np.sum(rho * V)
    expect = QE * w * (n_i - n_e)
    assert abs(total - expect) <= 1e-9 * QE * w * (n_i + n_e)

    phi = ctx.field(lib.FIELD_PHI)
    E = ctx.field(lib.FIELD_E)
    Eo = orc.electric_field(phi, DX, DX)
    assert np.max(np.abs(E - Eo)) <= 1e-9 * np.max(np.abs(Eo))
    ctx.close()
