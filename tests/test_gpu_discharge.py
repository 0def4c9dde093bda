"""Whole-loop statistical parity on a capacitively coupled argon discharge (a
small version of the RF-discharge configuration): electron and ion MCC, an
electrode driven at 300 V / 13.56 MHz the way problem/11_rf_discharge.jl does
it (apply_dirichlet with V(t) from the iteration hook), the other grounded,
discard! in x, wrap! in y.  The GPU runs iskra_step (one CUDA graph per
step); the oracle runs the reference's loop body (PicOracle) from the same
initial state with its own random stream.  Compared: accepted collisions per
process (3.5σ), surviving particle counts and the electron energy
distribution.

The GPU run carries 4x the oracle's macroparticles (weight / 4, the same
densities), so the oracle's sample dominates the statistical noise.  EEDF
agreement is stated as the L1 distance between the normalised electron
energy histograms (16 bins of 2.5 eV on 0-40 eV) and asserted below 0.02
(the configuration's "EEDF within 2 %"); the L1 expected from sampling
noise alone, Σ sqrt(2/π) sqrt(p (1-p) (1/n_g + 1/n_o)), is ~0.011 here."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QE = 1.602176634e-19
ME = 9.1093837015e-31
AMU = 1.66053906660e-27
KB = 1.380649e-23
EPS0 = 8.8541878128e-12
M_AR = 39.948 * AMU


def argon_tables(ne=1024):
    """Synthetic tables on 1024 log-spaced energies (0.01-1000 eV)."""
    eps = np.logspace(-2, 3, ne)
    el = np.full(ne, 1e-19)
    ex = np.where(eps > 11.5, np.minimum((eps - 11.5) / (100.0 - 11.5), 1.0) * 3e-21, 0.0)
    iz = np.where(eps > 15.76, 3e-20 * np.log(eps / 15.76) / np.log(100 / 15.76) * np.sqrt(100 / eps), 0.0)
    cx = np.full(ne, 5e-19)
    return eps, el, ex, iz, cx


def test_ccp_discharge_statistics(orc, lib):
    from iskra_gb300.device import Context

    nx, ny, gap = 129, 2, 0.025
    dx = gap / (nx - 1)
    n0, ng0 = 100000, 400000   # oracle / GPU macroparticles per species
    rng = np.random.default_rng(33)
    w = 1e15 * gap * dx / n0
    wg = 1e15 * gap * dx / ng0
    r = n0 / ng0               # GPU counts -> oracle scale

    def maxwellian(n, T_ev, m):
        x = np.column_stack([rng.uniform(0, gap, n), rng.uniform(0, dx, n)])
        v = rng.standard_normal((n, 3)) * np.sqrt(2 * T_ev * QE / m)
        return np.asfortranarray(x), np.asfortranarray(v)

    xe, ve = maxwellian(n0, 4.0, ME)
    xi, vi = maxwellian(n0, 0.03, M_AR)
    xeg, veg = maxwellian(ng0, 4.0, ME)
    xig, vig = maxwellian(ng0, 0.03, M_AR)
    eps, el, ex, iz, cx = argon_tables()
    gas_n = np.full((nx, ny), 3.0 / (KB * 300.0))
    dt = 7.4e-11
    steps = 400
    amp, f = 300.0, 13.56e6
    left = np.zeros((nx, ny), bool); left[0, :] = True
    right = np.zeros((nx, ny), bool); right[-1, :] = True

    # ---- GPU ----
    ctx = Context(nx, ny, dx, dx)
    se = ctx.species_create(-QE, ME, wg, 4 * ng0)
    si = ctx.species_create(QE, M_AR, wg, 4 * ng0)
    for s in (se, si):
        ctx.set_boundary(s, lib.BND_DISCARD, lib.BND_WRAP)
    ctx.upload(se, xeg, veg)
    ctx.upload(si, xig, vig)
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    ctx.apply_dirichlet(left, 0.0)
    ctx.apply_dirichlet(right, 0.0)
    ctx.drive_dirichlet(left, amp, f)
    assert ctx.set_method(0) == 0  # separable: the step runs as a CUDA graph
    me_, _ = ctx.mcc_create(se, [(lib.MCC_ELASTIC_ISOTROPIC, 0.0, eps, el), (lib.MCC_EXCITATION, 11.5, eps, ex),
                                 (lib.MCC_IONIZATION, 15.76, eps, iz)], M_AR, 300.0, gas_n, product=si)
    mi_, _ = ctx.mcc_create(si, [(lib.MCC_ELASTIC_BACKWARD, 0.0, eps, cx)], M_AR, 300.0, gas_n)
    ctx.set_sort_every(8)
    ctx.step(dt, steps, seed=5, rtol=1e-10)
    ctx.sync()
    cg = np.array(ctx.mcc_counts(me_, 3) + ctx.mcc_counts(mi_, 1), float)
    xe_g, ve_g, _ = ctx.download(se)
    ni_g = ctx.count(si)
    phi_g = ctx.field(lib.FIELD_PHI)
    ctx.close()

    # ---- oracle ----
    po = orc.PicOracle(nx, ny, dx, dx, EPS0)
    ie = po.add_species(-QE, ME, w, 4 * n0, xe, ve, bnd=(2, 1))
    ii = po.add_species(QE, M_AR, w, 4 * n0, xi, vi, bnd=(2, 1))
    po.ps.apply_periodic(1)
    po.ps.apply_dirichlet(left, 0.0)
    po.ps.apply_dirichlet(right, 0.0)
    po.drive_dirichlet(left, amp, f)
    po.add_mcc(orc.MCCOracle([("elastic_isotropic", 0.0, eps, el), ("excitation", 11.5, eps, ex),
                              ("ionization", 15.76, eps, iz)], ME, -QE, w, M_AR, 300.0, product_w0=w), ie, ii, gas_n)
    po.add_mcc(orc.MCCOracle([("elastic_backward", 0.0, eps, cx)], M_AR, QE, w, M_AR, 300.0), ii, None, gas_n)
    for s in range(steps):
        po.step(dt, 1000 + s)
    co = np.concatenate([po.counts[0], po.counts[1]]).astype(float)

    for k in range(4):
        sd = np.sqrt(r * r * cg[k] + co[k]) + 1.0
        assert abs(r * cg[k] - co[k]) <= 3.5 * sd, f"process {k}: gpu {cg[k]} (x{r}) oracle {co[k]}"
    ne_o, ni_o = po.species[ie].np, po.species[ii].np
    assert abs(r * len(xe_g) - ne_o) <= 0.03 * ne_o, (len(xe_g), ne_o)
    assert abs(r * ni_g - ni_o) <= 0.03 * ni_o, (ni_g, ni_o)
    # the driven electrode holds V((n-2)Δt) in both
    assert abs(phi_g[0, 0] - po.phi[0, 0]) <= 1e-9 * amp
    # electron energy distribution: the two runs draw different random
    # streams, so their EEDFs are two samples of one distribution.  Two-sample
    # chi-square (bins with fewer than 10 pooled counts merged), and the L1
    # distance, stated and below 2 %, beside its null expectation
    # Σ sqrt(2/π) sqrt(p (1-p) (1/n_g + 1/n_o)).
    bins = np.linspace(0.0, 40.0, 17)
    eg = 0.5 * ME * np.sum(ve_g ** 2, axis=1) / QE
    eo = 0.5 * ME * np.sum(po.species[ie].v[:ne_o] ** 2, axis=1) / QE
    cg_h = np.histogram(eg, bins)[0].astype(float)
    co_h = np.histogram(eo, bins)[0].astype(float)
    ng, no = cg_h.sum(), co_h.sum()
    p = (cg_h + co_h) / (ng + no)
    l1 = np.abs(cg_h / ng - co_h / no).sum()
    l1_null = np.sum(np.sqrt(2 / np.pi) * np.sqrt(p * (1 - p) * (1 / ng + 1 / no)))
    merged_g, merged_o, acc_g, acc_o = [], [], 0.0, 0.0
    for a, b in zip(cg_h, co_h):
        acc_g += a
        acc_o += b
        if acc_g + acc_o >= 10:
            merged_g.append(acc_g)
            merged_o.append(acc_o)
            acc_g = acc_o = 0.0
    merged_g[-1] += acc_g
    merged_o[-1] += acc_o
    from scipy.stats import chi2_contingency
    pval = chi2_contingency(np.array([merged_g, merged_o]))[1]
    print(f"EEDF L1 {l1:.4f} (sampling-noise expectation {l1_null:.4f}), chi2 p={pval:.2e}; "
          f"electrons gpu {len(xe_g)} (x{r}) oracle {ne_o}")
    assert l1 < 0.02, f"EEDF L1 {l1:.4f} (null {l1_null:.4f})"
    assert pval > 1e-4, f"EEDF chi2 p={pval:.2e}"
