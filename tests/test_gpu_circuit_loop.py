"""The RF-discharge configuration with its series RLC circuit in the loop:
electrode 1 (column i = 1) is a floating electrode (σ dof, apply_neumann in
its Gauss-law form) driven at 300 V / 13.56 MHz through R = 50 Ω, L = 1 µH,
C = 1 nF (advance!(::CircuitRLC), circuit_coupling.jl:35-43 ->
advance_circuit!, Circuit.jl:117-136); electrode 2 (column i = nx) is
grounded; electrons absorbed at electrode 1 credit its σ (hit!,
circuit_coupling.jl:45-55).  The GPU runs iskra_step (the circuit inside the
step graph); the oracle runs PicOracle with set_circuit from the same
initial particles.

Tolerances (each quantity's largest |difference| over the run, divided by
its largest |value| over the run):
  * no collisions, 300 steps: i, q, σ and ϕ at the driven node within 1e-2.
    FP32 push against the FP64 oracle: one macroparticle absorbed a step
    earlier or later moves σ by 6.4e-4 of its range; two oracle runs whose
    initial velocities differ by 1e-7 relative differ by at most 6.5e-4 (σ)
    and 1.1e-4 (i, ϕ).
  * with electron and ion MCC, 400 steps: i within 0.10, q within 0.04, σ
    within 0.08, ϕ within 0.04, accepted collisions per process within 3σ.
    The random streams differ, so these are statistical: oracle runs with
    four different seeds differ pairwise by at most 0.041 (i), 0.013 (q),
    0.034 (σ) and 0.012 (ϕ).
"""
import numpy as np
import pytest

from test_gpu_discharge import EPS0, KB, M_AR, ME, QE, argon_tables

pytestmark = pytest.mark.gpu

NX, NY, GAP = 129, 2, 0.025
DX = GAP / (NX - 1)
DT = 7.4e-11
R_, L_, C_, AMP, FREQ = 50.0, 1e-6, 1e-9, 300.0, 13.56e6


def initial_state(n0):
    rng = np.random.default_rng(33)

    def maxwellian(n, T_ev, m):
        x = np.column_stack([rng.uniform(0, GAP, n), rng.uniform(0, DX, n)])
        v = rng.standard_normal((n, 3)) * np.sqrt(2 * T_ev * QE / m)
        return np.asfortranarray(x), np.asfortranarray(v)

    return maxwellian(n0, 4.0, ME), maxwellian(n0, 0.03, M_AR)


def electrodes():
    left = np.zeros((NX, NY), bool)
    left[0, :] = True
    right = np.zeros((NX, NY), bool)
    right[-1, :] = True
    return left, right


def run_gpu(lib, n0, steps, mcc):
    from iskra_gb300.device import Context
    (xe, ve), (xi, vi) = initial_state(n0)
    w = 1e15 * GAP * DX / n0
    left, right = electrodes()
    ctx = Context(NX, NY, DX, DX)
    se = ctx.species_create(-QE, ME, w, 4 * n0)
    si = ctx.species_create(QE, M_AR, w, 4 * n0)
    for s in (se, si):
        ctx.set_boundary(s, lib.BND_DISCARD, lib.BND_WRAP)
    ctx.upload(se, xe, ve)
    ctx.upload(si, xi, vi)
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    dof = ctx.add_dof()
    ctx.apply_neumann(left, dof, gauss=True)
    ctx.apply_dirichlet(right, 0.0)
    ctx.circuit_create(R_, L_, C_, AMP, FREQ, 0.0, dof, left, right, DX * 1.0, 1.0)
    assert ctx.set_method(0) == 0  # separable: the step (with the circuit) runs as a CUDA graph
    mids = []
    if mcc:
        eps, el, ex, iz, cx = argon_tables()
        gas_n = np.full((NX, NY), 3.0 / (KB * 300.0))
        mids.append(ctx.mcc_create(se, [(lib.MCC_ELASTIC_ISOTROPIC, 0.0, eps, el), (lib.MCC_EXCITATION, 11.5, eps, ex),
                                        (lib.MCC_IONIZATION, 15.76, eps, iz)], M_AR, 300.0, gas_n, product=si)[0])
        mids.append(ctx.mcc_create(si, [(lib.MCC_ELASTIC_BACKWARD, 0.0, eps, cx)], M_AR, 300.0, gas_n)[0])
    hist = []
    for _ in range(steps):
        ctx.step(DT, 1, seed=5, rtol=1e-10)
        st = ctx.circuit_state()
        phi = ctx.field(lib.FIELD_PHI)
        hist.append((st["i"], st["q"], st["sigma"], phi[0, 0]))
    counts = np.array(ctx.mcc_counts(mids[0], 3) + ctx.mcc_counts(mids[1], 1), float) if mcc else None
    ne, ni = ctx.count(se), ctx.count(si)
    ctx.close()
    return np.array(hist), counts, (ne, ni)


def run_oracle(orc, n0, steps, mcc):
    (xe, ve), (xi, vi) = initial_state(n0)
    w = 1e15 * GAP * DX / n0
    left, right = electrodes()
    po = orc.PicOracle(NX, NY, DX, DX, EPS0)
    ie = po.add_species(-QE, ME, w, 4 * n0, xe, ve, bnd=(2, 1))
    ii = po.add_species(QE, M_AR, w, 4 * n0, xi, vi, bnd=(2, 1))
    po.ps.apply_periodic(1)
    dof = po.ps.add_new_dof()
    po.ps.apply_neumann(left, dof, gauss=True)
    po.ps.apply_dirichlet(right, 0.0)
    po.set_circuit(R_, L_, C_, AMP, FREQ, 0.0, dof, (0, 0), (NX - 1, 0), DX * 1.0)
    if mcc:
        eps, el, ex, iz, cx = argon_tables()
        gas_n = np.full((NX, NY), 3.0 / (KB * 300.0))
        po.add_mcc(orc.MCCOracle([("elastic_isotropic", 0.0, eps, el), ("excitation", 11.5, eps, ex),
                                  ("ionization", 15.76, eps, iz)], ME, -QE, w, M_AR, 300.0, product_w0=w),
                   ie, ii, gas_n)
        po.add_mcc(orc.MCCOracle([("elastic_backward", 0.0, eps, cx)], M_AR, QE, w, M_AR, 300.0), ii, None, gas_n)
    hist = []
    for s in range(steps):
        po.step(DT, 1000 + s)
        hist.append((po.circuit["state"][0], po.circuit["state"][1], po.ps.sig_b[dof - 1], po.phi[0, 0]))
    counts = np.concatenate(po.counts).astype(float) if mcc else None
    return np.array(hist), counts, (po.species[ie].np, po.species[ii].np)


def rel_dev(g, o):
    return [float(np.max(np.abs(g[:, k] - o[:, k])) / np.max(np.abs(o[:, k]))) for k in range(4)]


def test_circuit_loop_collisionless_matches_oracle(orc, lib):
    g, _, (ne, ni) = run_gpu(lib, 20000, 300, mcc=False)
    o, _, (ne_o, ni_o) = run_oracle(orc, 20000, 300, mcc=False)
    d = rel_dev(g, o)
    print(f"circuit loop (no MCC): max rel dev i {d[0]:.2e} q {d[1]:.2e} sigma {d[2]:.2e} phi {d[3]:.2e}; "
          f"e- {ne}/{ne_o} ions {ni}/{ni_o}")
    # the circuit really drives the electrode: ϕ reaches the source amplitude range
    assert np.max(np.abs(o[:, 3])) > 100.0
    assert max(d) <= 1e-2, d
    assert abs(ne - ne_o) <= 0.005 * ne_o + 2 and abs(ni - ni_o) <= 0.005 * ni_o + 2


def test_circuit_loop_with_mcc_statistics(orc, lib):
    g, cg, (ne, ni) = run_gpu(lib, 20000, 400, mcc=True)
    o, co, (ne_o, ni_o) = run_oracle(orc, 20000, 400, mcc=True)
    d = rel_dev(g, o)
    print(f"circuit loop (MCC): max rel dev i {d[0]:.3f} q {d[1]:.3f} sigma {d[2]:.3f} phi {d[3]:.3f}; "
          f"counts gpu {cg.tolist()} oracle {co.tolist()}")
    assert d[0] <= 0.10 and d[1] <= 0.04 and d[2] <= 0.08 and d[3] <= 0.04, d
    for k in range(4):
        sd = np.sqrt(cg[k] + co[k]) + 1.0
        assert abs(cg[k] - co[k]) <= 3 * sd, f"process {k}: gpu {cg[k]} oracle {co[k]}"
    assert abs(ne - ne_o) <= 0.03 * ne_o and abs(ni - ni_o) <= 0.03 * ni_o
