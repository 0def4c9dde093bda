"""Batched ensembles (the C4 configuration in small): R independent runs of a
capacitively coupled argon discharge in one ensemble, each compared with an
unbatched single-run context given the same initial particles, MCC seed and
drive amplitude.

* first step: the same particles and the same ρ bit for bit (integer
  deposit, same MCC keys), ϕ within FP64 rounding (direct FP64 solve against
  the iterative single-run solve), second-step particles within FP32 rounding;
* many steps, run by run: accepted collisions per process within 3.5σ,
  surviving counts within 3 %, electron energy distributions compatible
  (two-sample χ²)."""
import numpy as np
import pytest

from test_gpu_discharge import EPS0, KB, M_AR, ME, QE, argon_tables

pytestmark = pytest.mark.gpu

NX, NY, GAP = 129, 2, 0.025
DX = GAP / (NX - 1)
DT = 7.4e-11
FREQ = 13.56e6


def initial_state(seed, n0):
    rng = np.random.default_rng(seed)

    def maxwellian(n, T_ev, m):
        x = np.column_stack([rng.uniform(0, GAP, n), rng.uniform(0, DX, n)])
        v = rng.standard_normal((n, 3)) * np.sqrt(2 * T_ev * QE / m)
        return np.asfortranarray(x), np.asfortranarray(v)

    return maxwellian(n0, 4.0, ME), maxwellian(n0, 0.03, M_AR)


def configure(lib, n0, amp, w, mcc=True):
    """A single-run context set up like problem/11_rf_discharge.jl (driven
    Dirichlet electrode, grounded electrode, e- and Ar+ MCC unless mcc is
    False)."""
    from iskra_gb300.device import Context
    ctx = Context(NX, NY, DX, DX)
    se = ctx.species_create(-QE, ME, w, 4 * n0)
    si = ctx.species_create(QE, M_AR, w, 4 * n0)
    for s in (se, si):
        ctx.set_boundary(s, lib.BND_DISCARD, lib.BND_WRAP)
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    left = np.zeros((NX, NY), bool)
    left[0, :] = True
    right = np.zeros((NX, NY), bool)
    right[-1, :] = True
    ctx.apply_dirichlet(left, 0.0)
    ctx.apply_dirichlet(right, 0.0)
    ctx.drive_dirichlet(left, amp, FREQ)
    assert ctx.set_method(0) == 0
    if not mcc:
        return ctx, se, si, None, None
    eps, el, ex, iz, cx = argon_tables()
    gas_n = np.full((NX, NY), 3.0 / (KB * 300.0))
    me_, _ = ctx.mcc_create(se, [(lib.MCC_ELASTIC_ISOTROPIC, 0.0, eps, el), (lib.MCC_EXCITATION, 11.5, eps, ex),
                                 (lib.MCC_IONIZATION, 15.76, eps, iz)], M_AR, 300.0, gas_n, product=si)
    mi_, _ = ctx.mcc_create(si, [(lib.MCC_ELASTIC_BACKWARD, 0.0, eps, cx)], M_AR, 300.0, gas_n)
    return ctx, se, si, me_, mi_


def eedf_compatible(ve_a, ve_b):
    from scipy.stats import chi2_contingency
    bins = np.linspace(0.0, 40.0, 33)
    ea = 0.5 * ME * np.sum(ve_a ** 2, axis=1) / QE
    eb = 0.5 * ME * np.sum(ve_b ** 2, axis=1) / QE
    ha = np.histogram(ea, bins)[0].astype(float)
    hb = np.histogram(eb, bins)[0].astype(float)
    mg, mo, ag, ao = [], [], 0.0, 0.0
    for a, b in zip(ha, hb):
        ag += a
        ao += b
        if ag + ao >= 10:
            mg.append(ag)
            mo.append(ao)
            ag = ao = 0.0
    mg[-1] += ag
    mo[-1] += ao
    return chi2_contingency(np.array([mg, mo]))[1]


def make_ensemble(lib, R, n0, amps, mcc=True):
    from iskra_gb300.device import Ensemble
    w = 1e15 * GAP * DX / n0
    tmpl, se, si, me_, mi_ = configure(lib, n0, amps[0], w, mcc)
    ens = Ensemble(tmpl, R, 4 * n0)
    ens.set_seeds([1000 + r for r in range(R)])
    ens.set_drive_amplitude(0, np.asarray(amps, float))
    states = [initial_state(50 + r, n0) for r in range(R)]
    for r, ((xe, ve), (xi, vi)) in enumerate(states):
        ens.upload(r, se, xe, ve)
        ens.upload(r, si, xi, vi)
    return tmpl, ens, states, (se, si, me_, mi_), w


def single_run(lib, n0, amp, w, state, seed, steps, mcc=True):
    ctx, se, si, me_, mi_ = configure(lib, n0, amp, w, mcc)
    (xe, ve), (xi, vi) = state
    ctx.upload(se, xe, ve)
    ctx.upload(si, xi, vi)
    ctx.step(DT, steps, seed=seed, rtol=1e-12)
    ctx.sync()
    return ctx, (se, si, me_, mi_)


def test_ensemble_first_steps_match_single_runs(lib):
    R, n0 = 3, 4000
    amps = [150.0, 300.0, 450.0]
    tmpl, ens, states, (se, si, me_, mi_), w = make_ensemble(lib, R, n0, amps)
    ens.step(DT, 1)
    ens.sync()
    for r in range(R):
        ctx, _ = single_run(lib, n0, amps[r], w, states[r], 1000 + r, 1)
        rho_s = ctx.field(lib.FIELD_RHO)
        rho_e = ens.field(r, lib.FIELD_RHO)
        assert np.array_equal(rho_s, rho_e), f"run {r}: ρ differs after one step"
        phi_s = ctx.field(lib.FIELD_PHI)
        phi_e = ens.field(r, lib.FIELD_PHI)
        assert np.max(np.abs(phi_s - phi_e)) <= 1e-9 * max(1.0, np.max(np.abs(phi_s)))
        for s in (se, si):
            # the initial particles (ids 1..n0) match exactly; ionisation
            # children take ids in warp order, so only their number is compared
            xs, vs, ids_s = ctx.download(s)
            xe, ve, ids_e = ens.download(r, s)
            assert len(ids_s) == len(ids_e)
            ks, ke = ids_s <= n0, ids_e <= n0
            o_s, o_e = np.argsort(ids_s[ks]), np.argsort(ids_e[ke])
            assert np.array_equal(ids_s[ks][o_s], ids_e[ke][o_e])
            assert np.array_equal(xs[ks][o_s], xe[ke][o_e]) and np.array_equal(vs[ks][o_s], ve[ke][o_e])
        assert ens.mcc_counts(r, me_, 3) == [int(c) for c in ctx.mcc_counts(me_, 3)]
        ctx.close()
    # a second step: the pushes read E formed from the two solvers' ϕ
    ens.step(DT, 1)
    ens.sync()
    for r in range(R):
        ctx, _ = single_run(lib, n0, amps[r], w, states[r], 1000 + r, 2)
        xs, vs, ids_s = ctx.download(se)
        xe, ve, ids_e = ens.download(r, se)
        ks, ke = ids_s <= n0, ids_e <= n0
        o_s, o_e = np.argsort(ids_s[ks]), np.argsort(ids_e[ke])
        assert np.array_equal(ids_s[ks][o_s], ids_e[ke][o_e])
        assert np.allclose(xs[ks][o_s], xe[ke][o_e], rtol=0, atol=1e-6 * GAP)
        assert np.allclose(vs[ks][o_s], ve[ke][o_e], rtol=1e-5, atol=1.0)
        ctx.close()
    ens.close()
    tmpl.close()


def test_ensemble_without_mcc_matches_single_runs(lib):
    """A collisionless ensemble (the push without the folded MCC selection):
    after one step ρ and every particle equal the single run's bit for bit;
    after three steps (the pushes read E from the two solvers' ϕ) positions
    and velocities agree to FP32 rounding."""
    R, n0 = 3, 4000
    amps = [120.0, 260.0, 480.0]
    tmpl, ens, states, (se, si, _, _), w = make_ensemble(lib, R, n0, amps, mcc=False)
    ens.step(DT, 1)
    ens.sync()
    for r in range(R):
        ctx, _ = single_run(lib, n0, amps[r], w, states[r], 1000 + r, 1, mcc=False)
        assert np.array_equal(ctx.field(lib.FIELD_RHO), ens.field(r, lib.FIELD_RHO)), f"run {r}: ρ differs"
        for s in (se, si):
            xs, vs, ids_s = ctx.download(s)
            xe, ve, ids_e = ens.download(r, s)
            o_s, o_e = np.argsort(ids_s), np.argsort(ids_e)
            assert np.array_equal(ids_s[o_s], ids_e[o_e])
            assert np.array_equal(xs[o_s], xe[o_e]) and np.array_equal(vs[o_s], ve[o_e])
        ctx.close()
    ens.step(DT, 2)
    ens.sync()
    for r in range(R):
        ctx, _ = single_run(lib, n0, amps[r], w, states[r], 1000 + r, 3, mcc=False)
        for s in (se, si):
            xs, vs, ids_s = ctx.download(s)
            xe, ve, ids_e = ens.download(r, s)
            o_s, o_e = np.argsort(ids_s), np.argsort(ids_e)
            assert np.array_equal(ids_s[o_s], ids_e[o_e])
            assert np.allclose(xs[o_s], xe[o_e], rtol=0, atol=1e-6 * GAP)
            assert np.allclose(vs[o_s], ve[o_e], rtol=1e-5, atol=1.0)
        ctx.close()
    ens.close()
    tmpl.close()


def test_ensemble_runs_match_single_runs_statistically(lib):
    R, n0, steps = 4, 10000, 300
    amps = [120.0, 250.0, 380.0, 500.0]
    tmpl, ens, states, (se, si, me_, mi_), w = make_ensemble(lib, R, n0, amps)
    ens.step(DT, steps)
    ens.sync()
    for r in range(R):
        ctx, _ = single_run(lib, n0, amps[r], w, states[r], 1000 + r, steps)
        cg = np.array(ens.mcc_counts(r, me_, 3) + ens.mcc_counts(r, mi_, 1), float)
        cs = np.array(ctx.mcc_counts(me_, 3) + ctx.mcc_counts(mi_, 1), float)
        for k in range(4):
            sd = np.sqrt(cg[k] + cs[k]) + 1.0
            assert abs(cg[k] - cs[k]) <= 3.5 * sd, f"run {r} process {k}: ensemble {cg[k]} single {cs[k]}"
        for s in (se, si):
            ne, ns_ = ens.count(r, s), ctx.count(s)
            assert abs(ne - ns_) <= 0.03 * ns_, (r, s, ne, ns_)
        _, ve_e, _ = ens.download(r, se)
        _, ve_s, _ = ctx.download(se)
        l1, l1_null = eedf_l1(ve_e, ve_s)
        print(f"ensemble run {r} vs single run: EEDF L1 {l1:.4f} (sampling noise {l1_null:.4f})")
        assert eedf_compatible(ve_e, ve_s) > 1e-4, f"run {r}: EEDFs differ"
        assert l1 < 2.5 * l1_null, f"run {r}: EEDF L1 {l1:.4f} (null {l1_null:.4f})"
        ctx.close()
    ens.close()
    tmpl.close()


def eedf_l1(ve_a, ve_b):
    """L1 distance between normalised electron energy histograms (16 bins of
    2.5 eV on 0-40 eV) and its sampling-noise expectation
    Σ sqrt(2/π) sqrt(p (1-p) (1/n_a + 1/n_b))."""
    bins = np.linspace(0.0, 40.0, 17)
    ha = np.histogram(0.5 * ME * np.sum(ve_a ** 2, axis=1) / QE, bins)[0].astype(float)
    hb = np.histogram(0.5 * ME * np.sum(ve_b ** 2, axis=1) / QE, bins)[0].astype(float)
    na, nb = ha.sum(), hb.sum()
    p = (ha + hb) / (na + nb)
    return np.abs(ha / na - hb / nb).sum(), np.sum(np.sqrt(2 / np.pi) * np.sqrt(p * (1 - p) * (1 / na + 1 / nb)))


def test_ensemble_runs_match_oracle(orc, lib):
    """Ensemble runs against the FP64 oracle's loop body (PicOracle) directly:
    two runs of the batched discharge (drive amplitudes 200 V and 400 V),
    400 steps, each ensemble run from the same initial particles as its
    oracle run (the same macroparticle count: with four times the particles
    at a quarter of the weight, the 400 V run's ionization and excitation
    counts fell 2.5-9 % below the oracle's, ~3σ, the smaller numerical
    heating of the finer sampling).  Per run: accepted collisions per
    process within 3.5σ, surviving counts within 3 %, EEDF L1 below 0.02
    (the configuration's 2 %; the sampling-noise expectation is printed)."""
    R, n0, steps = 2, 100000, 400
    amps = [200.0, 400.0]
    r_ = 1.0
    tmpl, ens, _, (se, si, me_, mi_), _ = make_ensemble(lib, R, n0, amps)
    for r in range(R):
        (xe, ve), (xi, vi) = initial_state(90 + r, n0)
        ens.upload(r, se, xe, ve)
        ens.upload(r, si, xi, vi)
    ens.step(DT, steps)
    ens.sync()
    eps, el, ex, iz, cx = argon_tables()
    gas_n = np.full((NX, NY), 3.0 / (KB * 300.0))
    left = np.zeros((NX, NY), bool)
    left[0, :] = True
    right = np.zeros((NX, NY), bool)
    right[-1, :] = True
    w = 1e15 * GAP * DX / n0
    for r in range(R):
        (xe, ve), (xi, vi) = initial_state(90 + r, n0)
        po = orc.PicOracle(NX, NY, DX, DX, EPS0)
        ie = po.add_species(-QE, ME, w, 4 * n0, xe, ve, bnd=(2, 1))
        ii = po.add_species(QE, M_AR, w, 4 * n0, xi, vi, bnd=(2, 1))
        po.ps.apply_periodic(1)
        po.ps.apply_dirichlet(left, 0.0)
        po.ps.apply_dirichlet(right, 0.0)
        po.drive_dirichlet(left, amps[r], FREQ)
        po.add_mcc(orc.MCCOracle([("elastic_isotropic", 0.0, eps, el), ("excitation", 11.5, eps, ex),
                                  ("ionization", 15.76, eps, iz)], ME, -QE, w, M_AR, 300.0, product_w0=w),
                   ie, ii, gas_n)
        po.add_mcc(orc.MCCOracle([("elastic_backward", 0.0, eps, cx)], M_AR, QE, w, M_AR, 300.0), ii, None, gas_n)
        for s in range(steps):
            po.step(DT, 7000 + 1000 * r + s)
        co = np.concatenate(po.counts).astype(float)
        cg = np.array(ens.mcc_counts(r, me_, 3) + ens.mcc_counts(r, mi_, 1), float)
        for k in range(4):
            sd = np.sqrt(r_ * r_ * cg[k] + co[k]) + 1.0
            assert abs(r_ * cg[k] - co[k]) <= 3.5 * sd, f"run {r} process {k}: ensemble {cg[k]} (x{r_}) oracle {co[k]}"
        for s, k in ((se, ie), (si, ii)):
            ne, no = ens.count(r, s), po.species[k].np
            assert abs(r_ * ne - no) <= 0.03 * no, (r, s, ne, no)
        _, ve_e, _ = ens.download(r, se)
        l1, l1_null = eedf_l1(ve_e, po.species[ie].v[:po.species[ie].np])
        print(f"ensemble run {r} ({amps[r]:.0f} V) vs oracle: EEDF L1 {l1:.4f} (sampling noise {l1_null:.4f}), "
              f"counts ensemble {cg.tolist()} (x{r_}) oracle {co.tolist()}")
        assert l1 < 0.02, f"run {r}: EEDF L1 {l1:.4f} (null {l1_null:.4f})"
        ph = ens.field(r, lib.FIELD_PHI)
        assert abs(ph[0, 0] - po.phi[0, 0]) <= 1e-9 * amps[r]  # the driven electrode, V((n-2)Δt)
    ens.close()
    tmpl.close()


def test_ensemble_field_solve_with_complex_modes(lib):
    """The ensemble's direct field solve (DFT along y + cyclic reduction per
    Fourier mode) on a 41 x 8 grid, y periodic (N = 8: modes 0..4, three of
    them complex): after one step ρ equals the single run's bit for bit and
    ϕ agrees to 1e-9 of its range, run by run."""
    from iskra_gb300.device import Context, Ensemble
    nx, ny, gap = 41, 8, 0.01
    dx = gap / (nx - 1)
    n0, R = 3000, 2
    amps = [150.0, 400.0]
    w = 1e15 * gap * dx * (ny - 1) / n0

    def context(amp):
        ctx = Context(nx, ny, dx, dx)
        se = ctx.species_create(-QE, ME, w, 4 * n0)
        si = ctx.species_create(QE, M_AR, w, 4 * n0)
        for s in (se, si):
            ctx.set_boundary(s, lib.BND_DISCARD, lib.BND_WRAP)
        ctx.poisson_create(EPS0)
        ctx.apply_periodic(1)
        left = np.zeros((nx, ny), bool)
        left[0, :] = True
        right = np.zeros((nx, ny), bool)
        right[-1, :] = True
        ctx.apply_dirichlet(left, 0.0)
        ctx.apply_dirichlet(right, 0.0)
        ctx.drive_dirichlet(left, amp, FREQ)
        assert ctx.set_method(0) == 0
        return ctx, se, si

    rng = np.random.default_rng(8)
    states = []
    for r in range(R):
        st = []
        for T, m in ((4.0, ME), (0.03, M_AR)):
            x = np.asfortranarray(np.column_stack([rng.uniform(0, gap, n0), rng.uniform(0, (ny - 1) * dx, n0)]))
            v = np.asfortranarray(rng.standard_normal((n0, 3)) * np.sqrt(2 * T * QE / m))
            st.append((x, v))
        states.append(st)
    tmpl, se, si = context(amps[0])
    ens = Ensemble(tmpl, R, 4 * n0)
    ens.set_drive_amplitude(0, np.asarray(amps, float))
    for r in range(R):
        for s, (x, v) in zip((se, si), states[r]):
            ens.upload(r, s, x, v)
    ens.step(DT, 1)
    ens.sync()
    for r in range(R):
        ctx, se1, si1 = context(amps[r])
        for s, (x, v) in zip((se1, si1), states[r]):
            ctx.upload(s, x, v)
        ctx.step(DT, 1, seed=1, rtol=1e-12)
        ctx.sync()
        assert np.array_equal(ctx.field(lib.FIELD_RHO), ens.field(r, lib.FIELD_RHO)), f"run {r}: ρ differs"
        ps, pe = ctx.field(lib.FIELD_PHI), ens.field(r, lib.FIELD_PHI)
        assert np.max(np.abs(ps - pe)) <= 1e-9 * max(1.0, np.max(np.abs(ps))), f"run {r}: ϕ differs"
        for s in (se1, si1):
            xs, vs, ids_s = ctx.download(s)
            xe, ve, ids_e = ens.download(r, s)
            o_s, o_e = np.argsort(ids_s), np.argsort(ids_e)
            assert np.array_equal(ids_s[o_s], ids_e[o_e])
            assert np.array_equal(xs[o_s], xe[o_e]) and np.array_equal(vs[o_s], ve[o_e])
        ctx.close()
    ens.close()
    tmpl.close()
