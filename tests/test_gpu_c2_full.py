"""One-step parity on the benchmarked configuration at its full size: the 2D XY
plasma slab, 512x512 nodes, 4M electrons + 4M Ar+ ions, x Dirichlet 0/100 V
with discard!, y wrap! (the workload bench.py times).  After three steps from
the seeded initial state (so E is the field of a developed step, not zero),
one more iskra_step is checked stage by stage against the FP64 oracle, each
stage from the device's own downloaded inputs:

  * push (gather + Boris + discard!/wrap!) of both species from the state
    before the step and its E (FP32, as the push reads it): the surviving id
    sets equal, positions and velocities within 1e-6 relative (the
    tolerances of tests/test_gpu_parity.py);
  * ρ from the device's pushed positions: within 1e-9 of max|ρ|;
  * ϕ and E after a solve to relative residual 1e-10: ϕ within 1e-7 of
    max|ϕ| of the oracle's sparse LU solve, E within 1e-6 of max|E|.
"""
import numpy as np
import pytest

import bench
from test_gpu_parity import by_id, check_push

pytestmark = pytest.mark.gpu


def test_slab_512_full_size_step_matches_oracle(orc, lib):
    w, e, i = bench.make_state()
    ctx, se, si = bench.setup_context(w, e, i)
    del e, i
    dt = bench.DT
    ctx.step(dt, 3, seed=0, rtol=1e-10)
    ctx.sync()
    before = [by_id(*ctx.download(s)) for s in (se, si)]
    E0 = ctx.field(lib.FIELD_E)
    ctx.step(dt, 1, seed=0, rtol=1e-10)
    ctx.sync()
    after = [by_id(*ctx.download(s)) for s in (se, si)]
    rho1 = ctx.field(lib.FIELD_RHO)
    phi1 = ctx.field(lib.FIELD_PHI)
    E1 = ctx.field(lib.FIELD_E)
    _, rr = ctx.solve_info()
    ctx.close()
    assert rr <= 1e-10
    nx, ny, dx = bench.NX, bench.NY, bench.DX
    assert np.max(np.abs(E0[:, :, :2])) > 1e3  # a developed field: the gather is exercised

    # push of both species from the device's state before the step
    E32 = E0.copy(order="F")
    E32[:, :, :2] = E0[:, :, :2].astype(np.float32)
    for (x0, v0, i0), (x1, v1, i1), qm in zip(before, after, (-bench.QE / bench.ME, bench.QE / bench.M_AR)):
        xr, vr = x0.copy(order="F"), v0.copy(order="F")
        pu = orc.grid_to_particle(E32, dx, dx, xr)
        orc.push_cartesian(xr, vr, pu, None, qm, dt)
        ids = i0.copy()
        npn, _, _ = orc.discard(xr, vr, np.full(len(xr), w), ids, w, 0, nx, dx)
        xr, vr, ids = np.asfortranarray(xr[:npn]), np.asfortranarray(vr[:npn]), ids[:npn].copy()
        orc.wrap(xr, 1, ny, dx)
        o = np.argsort(ids)
        assert np.array_equal(ids[o], i1), "surviving particle set differs"
        check_push(x1, v1, xr[o], vr[o], v0[np.searchsorted(i0, ids[o])], dx)
        del xr, vr, pu

    # ρ from the device's pushed positions
    rho_o = sum(q * orc.density(nx, ny, dx, dx, st[0], w, (0, 0, 0, 0))
                for q, st in ((-bench.QE, after[0]), (bench.QE, after[1])))
    assert np.max(np.abs(rho1 - rho_o)) <= 1e-9 * np.max(np.abs(rho_o))

    # ϕ and E: the reference's operator solved by the oracle's sparse LU
    ps = orc.PoissonOracle(nx, ny, dx, dx, bench.EPS0)
    ps.apply_periodic(1)
    left, right = bench.electrode_masks()
    ps.apply_dirichlet(left, 0.0)
    ps.apply_dirichlet(right, bench.V_RIGHT)
    phi_o = ps.solve(-rho_o)
    assert np.max(np.abs(phi1 - phi_o)) <= 1e-7 * np.max(np.abs(phi_o))
    E_o = orc.electric_field(phi_o, dx, dx)
    assert np.max(np.abs(E1 - E_o)) <= 1e-6 * np.max(np.abs(E_o))
