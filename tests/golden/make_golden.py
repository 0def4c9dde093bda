"""Generates tests/golden/oracle_fixtures.npz from the FP64 oracle.

The reference (Julia) cannot run in this environment and ships no fixtures, so
these vectors are produced by the oracle restatement itself: they pin the
oracle against regressions (tests/test_oracle_cpu.py recomputes and compares
bit for bit) while the analytic known-answer tests in the same file pin it to
the reference's mathematics.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as orc  # noqa: E402

QE = 1.602176634e-19
ME = 9.1093837015e-31
EPS0 = 8.8541878128e-12


def fixtures():
    out = {}
    rng = np.random.default_rng(20240611)
    nx, ny, dx, dy = 9, 6, 0.01, 0.02
    n = 64
    x = np.asfortranarray(np.column_stack([rng.uniform(0, (nx - 1) * dx, n), rng.uniform(0, (ny - 1) * dy, n)]))
    v = np.asfortranarray(rng.normal(0, 1e5, (n, 3)))
    E = np.asfortranarray(rng.normal(0, 1e3, (nx, ny, 3)))
    out["x0"], out["v0"], out["E"] = x, v, E
    pu = orc.grid_to_particle(E, dx, dy, x)
    out["gather"] = pu
    x1, v1 = x.copy(order="F"), v.copy(order="F")
    orc.push_cartesian(x1, v1, pu, None, -QE / ME, 2e-9)
    out["push_x"], out["push_v"] = x1.copy(), v1.copy()
    xw = x1.copy(order="F")
    orc.wrap(xw, 0, nx, dx)
    orc.wrap(xw, 1, ny, dy)
    out["wrap_x"] = xw
    xd, vd = x1.copy(order="F"), v1.copy(order="F")
    wg = np.full(n, 3.0)
    ids = np.arange(1, n + 1, dtype=np.uint32)
    npn, lo, hi = orc.discard(xd, vd, wg, ids, 3.0, 0, nx, dx)
    out["discard_n"] = np.array([npn, lo, hi])
    out["discard_ids"] = ids[:npn].copy()
    out["density"] = orc.density(nx, ny, dx, dy, xw, 7.0, (0, 1, 0, 0))
    ps = orc.PoissonOracle(nx, ny, dx, dx, EPS0)
    ps.apply_periodic(1)
    m1 = np.zeros((nx, ny), bool)
    m1[0, :] = True
    m2 = np.zeros((nx, ny), bool)
    m2[-1, :] = True
    ps.apply_dirichlet(m1, 0.0)
    ps.apply_dirichlet(m2, 5.0)
    rho = rng.normal(0, 1e-9, (nx, ny))
    out["rho"] = rho
    out["phi_slab"] = ps.solve(-rho)
    ps2 = orc.PoissonOracle(nx, ny, dx, dx, EPS0)
    ps2.apply_periodic(1)
    dof = ps2.add_new_dof()
    ps2.apply_neumann(m1, dof)
    ps2.set_sigma(dof, 2e-7)
    ps2.apply_dirichlet(m2, 0.0)
    out["phi_neumann"] = ps2.solve(-rho)
    out["A_neumann"] = ps2.matrix().toarray()
    out["efield"] = orc.electric_field(out["phi_slab"], dx, dx)
    st = np.zeros(3)
    traj = []
    for k in range(10):
        st = orc.advance_circuit(50.0, 1e-6, 1e-9, st, 0.3 * k, 300.0 * np.sin(2 * np.pi * 13.56e6 * st[2]), 7.4e-11)
        traj.append(st.copy())
    out["circuit"] = np.array(traj)
    eps = np.logspace(-2, 3, 16)
    sig = np.linspace(1e-20, 3e-20, 16)
    probes = np.array([0.001, 0.01, 0.5, 7.3, 999.0, 1000.0, 2000.0])
    out["sigma_probe"] = np.array([orc.sigma(eps, sig, e) for e in probes])
    vv = rng.normal(0, 1e6, (8, 3))
    uu = rng.uniform(0, 1, (8, 2))
    out["iso_in"], out["iso_u"] = vv, uu
    out["iso"] = np.array([orc.isotropic_scattering(vv[k], *uu[k]) for k in range(8)])
    out["diffuse"] = np.array([orc.diffuse_reflection(vv[k], *uu[k]) for k in range(8)])
    return out


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "oracle_fixtures.npz"), **fixtures())
    print("wrote", os.path.join(HERE, "oracle_fixtures.npz"))
