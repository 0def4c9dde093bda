"""The configuration of problem/07_boundaries.jl through the reference-named
Python mirror: a thermalized electron beam loaded by init (sources.jl), a
driven (floating, σ = ε0) wall electrode, a floating and a grounded
electrode, a reflective block (surfaces/*.jl, circuit_coupling.jl) and the
solve loop.  Checks what the tracker guarantees: no electron gets inside the
reflective block, every absorbed electron is counted on some surface and
the floating electrodes' σ moved by exactly q w / area per hit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QE, ME, EPS0, KB = 1.602176634e-19, 9.1093837015e-31, 8.8541878128e-12, 1.380649e-23


def test_07_boundaries(lib):
    from iskra_gb300 import finite_difference_method as fdm
    from iskra_gb300 import particle_in_cell as pic
    from iskra_gb300.regular_grids import create_uniform_grid

    nx = ny = 10
    dh, dt, ts = 0.1, 10e-9, 200
    Lx, Ly = nx * dh, ny * dh
    xs = np.arange(nx) * dh
    grid = create_uniform_grid(xs, xs)
    e = pic.create_kinetic_species("e-", 50_000, -QE, ME, 50e3, grid)
    config = pic.Config()
    config.grid = grid
    config.solver = fdm.create_poisson_solver(grid, EPS0)
    config.species = [e]
    # after_push = wrap! (the reference's default hook); the walls are
    # absorbing surfaces of the tracker, so nothing reaches wrap!
    pic.wrap(e, grid)
    bcs = np.zeros((nx, ny), np.int8)
    bcs[0, 1:ny - 1] = 1
    bcs[nx - 1, 4:7] = 2
    bcs[nx - 2, 0] = 3
    bcs[nx - 2, ny - 1] = 3
    bcs[5:8, 4:7] = 4
    driven = pic.create_electrode(bcs == 1, config, sigma=1 * EPS0)
    floating = pic.create_electrode(bcs == 2, config)
    grounded = pic.create_electrode(bcs == 3, config, fixed=True)
    reflecting = pic.create_reflective_surface()
    pic.track_surface(config.tracker, bcs == 4, reflecting)
    sig0 = {el: fdm.get_rhs(config.solver, "σ", el.dof) for el in (driven, floating)}

    beam = pic.create_thermalized_beam(e, [Lx / 4, Ly / 2], [0.0, 0.0, 0.0], dx=[Lx / 4, Lx / 4], T=300.0,
                                       rate=20_000 / dt)
    pic.init(beam, e, dt, seed=1)
    n0 = e.np
    assert n0 == int(np.floor(beam.rate * dt)) and 19_999 <= n0 <= 20_000
    pic.solve(config, dt, ts, seed=1, rtol=1e-8)

    x, v, ids = e.state()
    n = len(x)
    # the reflective block spans nodes 6..8 x 5..7 (1-based): x, y in [0.5, 0.7] x [0.4, 0.6]
    inside = (x[:, 0] > 0.5 + 1e-9) & (x[:, 0] < 0.7 - 1e-9) & (x[:, 1] > 0.4 + 1e-9) & (x[:, 1] < 0.6 - 1e-9)
    assert not inside.any()
    assert len(np.unique(ids)) == n
    tr = config.tracker
    hits = {s: tr.hits(s, e) for s in tr.surfaces}
    assert hits[reflecting] == 0
    assert sum(hits.values()) == n0 - n              # every lost electron hit a surface
    assert sum(hits.values()) > 0
    for el in (driven, floating):
        dsig = fdm.get_rhs(config.solver, "σ", el.dof) - sig0[el]
        assert np.isclose(dsig, -QE * 50e3 * hits[el] / el.area, rtol=1e-12, atol=1e-30)
    assert np.all(np.isfinite(v))
