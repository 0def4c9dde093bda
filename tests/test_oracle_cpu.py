"""CPU tests of the FP64 oracle: the reference's own known-answer test, analytic
known answers for each restated function, an independent literal restatement
of the Poisson assembly loops, and the committed regression fixtures."""
import os

import numpy as np
import pytest

QE = 1.602176634e-19
ME = 9.1093837015e-31
EPS0 = 8.8541878128e-12
HERE = os.path.dirname(os.path.abspath(__file__))


def test_parallel_capacitor_reference_kat(orc):
    """FiniteDifferenceMethod/test/runtests.jl:8-22 restated with the current
    API: grid 0:0.5:1 x 0:0.5:2, 0 V at column 1, 1 V at column 3."""
    nx, ny, dx = 3, 5, 0.5
    ps = orc.PoissonOracle(nx, ny, dx, dx, EPS0)
    bcs = np.zeros((nx, ny), dtype=np.int8)
    bcs[0, :] = 1
    bcs[2, :] = 2
    ps.apply_dirichlet(bcs == 1, 0.0)
    ps.apply_dirichlet(bcs == 2, 1.0)
    E = orc.electric_field(ps.solve(np.zeros((nx, ny))), dx, dx)
    assert np.allclose(E[:, :, 0], -1.0, rtol=np.sqrt(np.finfo(float).eps), atol=0)  # ≈ -1ones(3,5)
    assert np.linalg.norm(E[:, :, 1]) <= 1e-15                                         # ≈ zeros atol=1e-15


def test_particle_cell(orc):
    i, j, hx, hy = orc.particle_cell(0.25, 0.0, 0.1, 0.1)
    assert (i, j) == (3, 1) and abs(hx - 0.5) < 1e-12 and hy == 0.0


def test_free_streaming_and_uniform_field(orc):
    n = 100
    rng = np.random.default_rng(0)
    x = np.asfortranarray(rng.uniform(0, 1, (n, 2)))
    v = np.asfortranarray(rng.normal(0, 1e5, (n, 3)))
    x0, v0 = x.copy(), v.copy()
    orc.push_cartesian(x, v, np.zeros((n, 3)), None, -QE / ME, 1e-9)
    assert np.array_equal(v, v0)
    assert np.allclose(x, x0 + 1e-9 * v0[:, :2], rtol=1e-15, atol=0)
    x, v = x0.copy(order="F"), v0.copy(order="F")
    E = np.zeros((n, 3))
    E[:, 0] = 1e3
    orc.push_cartesian(x, v, E, None, -QE / ME, 1e-9)
    assert np.allclose(v[:, 0] - v0[:, 0], -QE / ME * 1e3 * 1e-9, rtol=1e-12)
    assert np.array_equal(v[:, 1:], v0[:, 1:])


def test_cic_partition_of_unity_and_bilinear_exactness(orc):
    nx, ny, dx, dy = 7, 5, 0.1, 0.2
    rng = np.random.default_rng(1)
    x = np.asfortranarray(np.column_stack([rng.uniform(0, 0.6, 50), rng.uniform(0, 0.8, 50)]))
    u = orc.particle_to_grid(nx, ny, dx, dy, x, None, 2.5)
    assert abs(u.sum() - 50 * 2.5) < 1e-12
    I, J = np.meshgrid(np.arange(nx) * dx, np.arange(ny) * dy, indexing="ij")
    E = np.zeros((nx, ny, 3), order="F")
    E[:, :, 0] = 3 + 2 * I - 5 * J + 7 * I * J
    pu = orc.grid_to_particle(E, dx, dy, x)
    exact = 3 + 2 * x[:, 0] - 5 * x[:, 1] + 7 * x[:, 0] * x[:, 1]
    assert np.allclose(pu[:, 0], exact, rtol=1e-12, atol=1e-12)


def test_wrap_semantics(orc):
    n_nodes, dh = 11, 0.1
    L = (n_nodes - 1) * dh
    x = np.asfortranarray(np.array([[L + 0.05, 0], [-0.05, 0], [np.nextafter(L, 0), 0], [0.0, 0], [2 * L + 0.01, 0]]))
    orc.wrap(x, 0, n_nodes, dh)
    assert abs(x[0, 0] - 0.05) < 1e-12 and abs(x[1, 0] - (L - 0.05)) < 1e-12
    assert x[2, 0] == np.nextafter(L, 0) and x[3, 0] == 0.0 and abs(x[4, 0] - 0.01) < 1e-12


def test_discard_matches_literal_julia_loop(orc):
    """discard! iterates p = np..1 and swap-removes (wrap.jl:1-18, kinetic.jl:20-27)."""
    rng = np.random.default_rng(3)
    n, n_nodes, dh = 40, 6, 0.2
    x = np.asfortranarray(np.column_stack([rng.uniform(-0.3, 1.3, n), rng.uniform(0, 1, n)]))
    v = np.asfortranarray(rng.normal(size=(n, 3)))
    ids = np.arange(1, n + 1, dtype=np.uint32)
    wg = np.full(n, 2.0)
    # literal restatement
    xl, vl, il, np_ = x.copy(), v.copy(), ids.copy(), n
    L = (n_nodes - 1) * dh
    for p in range(n - 1, -1, -1):
        if np.floor(xl[p, 0] / L) != 0:
            last = np_ - 1
            xl[p], vl[p] = xl[last].copy(), vl[last].copy()
            il[p], il[last] = il[last], il[p]
            np_ -= 1
    npn, lo, hi = orc.discard(x, v, wg, ids, 2.0, 0, n_nodes, dh)
    assert npn == np_
    assert np.array_equal(ids[:npn], il[:np_]) and np.array_equal(x[:npn], xl[:np_])
    assert lo + hi == n - npn


def test_cell_volume_and_mirror(orc):
    from iskra_gb300.regular_grids import cell_volume, create_uniform_grid
    g = create_uniform_grid(np.arange(6) * 0.1, np.arange(4) * 0.2, bottom="periodic", top="periodic")
    V = cell_volume(g)
    Vo = orc.cell_volume(6, 4, 0.1, 0.2, (0, 0, 1, 1))
    assert np.allclose(V, Vo, rtol=1e-15)
    assert V[0, 1] == 0.5 * 0.1 * 0.2 and V[2, 0] == 0.1 * 0.2


def _literal_poisson(nx, ny, dh, periodic_axes, dirichlet, neumann):
    """Dense literal restatement of generalized_poisson.jl's loops (1-based)."""
    nn = nx * ny
    A = np.zeros((nn, nn))
    phi = lambda i, j: (i - 1) + nx * (j - 1)  # noqa: E731
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            if i < nx:
                A[phi(i, j), phi(i, j)] -= 1; A[phi(i, j), phi(i + 1, j)] += 1
            if i > 1:
                A[phi(i, j), phi(i, j)] -= 1; A[phi(i, j), phi(i - 1, j)] += 1
            if j < ny:
                A[phi(i, j), phi(i, j)] -= 1; A[phi(i, j), phi(i, j + 1)] += 1
            if j > 1:
                A[phi(i, j), phi(i, j)] -= 1; A[phi(i, j), phi(i, j - 1)] += 1
    A /= dh ** 2
    for axis in periodic_axes:
        if axis == 1:
            for j in (1, ny):
                for i in range(1, nx + 1):
                    if j == ny:
                        A[phi(i, j), phi(i, j)] -= 1 / dh ** 2; A[phi(i, j), phi(i, 1)] += 1 / dh ** 2
                    if j == 1:
                        A[phi(i, j), phi(i, j)] -= 1 / dh ** 2; A[phi(i, j), phi(i, ny)] += 1 / dh ** 2
        else:
            for j in range(1, ny + 1):
                for i in (1, nx):
                    if i == nx:
                        A[phi(i, j), phi(i, j)] -= 1 / dh ** 2; A[phi(i, j), phi(1, j)] += 1 / dh ** 2
                    if i == 1:
                        A[phi(i, j), phi(i, j)] -= 1 / dh ** 2; A[phi(i, j), phi(nx, j)] += 1 / dh ** 2
    nsig = 1 if neumann is not None else 0
    A = np.pad(A, ((0, nsig), (0, nsig)))
    if nsig:
        A[nn, nn] = 1
    for mask, _ in dirichlet:
        for (i0, j0) in zip(*np.nonzero(mask)):
            A[phi(i0 + 1, j0 + 1), :] = 0
            A[phi(i0 + 1, j0 + 1), phi(i0 + 1, j0 + 1)] = 1
    if neumann is not None:
        for (i0, j0) in zip(*np.nonzero(neumann)):
            i, j = i0 + 1, j0 + 1
            a = neumann[i0 - 1, j0] if i > 1 else False
            b = neumann[i0 + 1, j0] if i < nx else False
            c = neumann[i0, j0 - 1] if j > 1 else True
            d = neumann[i0, j0 + 1] if j < ny else True
            if c == d == True and a == b == False:  # noqa: E712
                ip = i + 1 if i == 1 else i - 1
                A[phi(i, j), :] = 0
                A[phi(i, j), phi(i, j)] -= 2 / dh
                A[phi(i, j), phi(ip, j)] += 2 / dh
                A[phi(i, j), nn] += 2
    return A


@pytest.mark.parametrize("case", ["slab", "periodic", "neumann", "ny2"])
def test_poisson_assembly_matches_literal_loops(orc, case):
    nx, ny, dh = 6, 4 if case != "ny2" else 2, 0.1
    m1 = np.zeros((nx, ny), bool); m1[0, :] = True
    m2 = np.zeros((nx, ny), bool); m2[-1, :] = True
    ps = orc.PoissonOracle(nx, ny, dh, dh, EPS0)
    if case in ("slab", "ny2"):
        axes, dirich, neu = (1,), [(m1, 0.0), (m2, 1.0)], None
    elif case == "periodic":
        axes, dirich, neu = (1, 2), [], None
    else:
        axes, dirich, neu = (1,), [(m2, 0.0)], m1
    for a in axes:
        ps.apply_periodic(a)
    if neu is not None:
        dof = ps.add_new_dof()
        ps.apply_neumann(neu, dof)
    for m, val in dirich:
        ps.apply_dirichlet(m, val)
    A_lit = _literal_poisson(nx, ny, dh, axes, dirich, neu)
    assert np.allclose(ps.matrix().toarray(), A_lit, rtol=0, atol=1e-9 * np.abs(A_lit).max())


def test_periodic_poisson_gauge_and_field(orc):
    nx, ny, dh = 16, 2, 0.05
    ps = orc.PoissonOracle(nx, ny, dh, dh, EPS0)
    ps.apply_periodic(1)
    ps.apply_periodic(2)
    rng = np.random.default_rng(4)
    rho = rng.normal(size=(nx, ny))
    rho -= rho.mean()
    phi = ps.solve(-rho)
    assert abs(phi.mean()) < 1e-9 * np.abs(phi).max()
    assert ps.residual(phi, -rho) < 1e-12


def test_circuit_recurrence(orc):
    """advance_circuit! (Circuit.jl:117-136) restated literally."""
    R, L, C, dt = 50.0, 1e-6, 1e-9, 7.4e-11
    st = np.zeros(3)
    i = q = t = 0.0
    for k in range(20):
        vsrc = 300 * np.sin(2 * np.pi * 13.56e6 * t)
        st = orc.advance_circuit(R, L, C, st, 0.0, vsrc, dt)
        inew = ((L / dt - R / 2) * i + 0.0 - vsrc - q / C) / (L / dt + R / 2)
        q, i, t = q + dt * i, inew, t + dt
        assert st[0] == inew and st[1] == q and st[2] == t


def test_lc_oscillation_frequency(orc):
    """R = 0, V = 0: the recurrence oscillates at ~1/sqrt(LC)."""
    L, C = 1e-6, 1e-9
    dt = 2 * np.pi * np.sqrt(L * C) / 2000
    st = np.array([0.0, 1e-9, 0.0])
    qs = []
    for k in range(4000):
        st = orc.advance_circuit(0.0, L, C, st, 0.0, 0.0, dt)
        qs.append(st[1])
    qs = np.array(qs)
    zc = np.nonzero(np.diff(np.sign(qs)))[0]
    period = 2 * np.mean(np.diff(zc)) * dt
    assert abs(period - 2 * np.pi * np.sqrt(L * C)) < 0.01 * period


def test_cross_section_interpolation(orc):
    e = np.array([1.0, 2.0, 4.0])
    s = np.array([10.0, 20.0, 0.0])
    assert orc.sigma(e, s, 0.5) == 10.0 and orc.sigma(e, s, 9.0) == 0.0
    assert orc.sigma(e, s, 2.0) == 20.0 and abs(orc.sigma(e, s, 3.0) - 10.0) < 1e-14
    assert abs(orc.sigma(e, s, 1.5) - 15.0) < 1e-14


def _literal_rotation(v, sch, cch, seta, ceta):
    """[sinχcosη sinχsinη cosχ] * unrotated(θ, ϕ) literally (mcc.jl:83-113)."""
    nv = np.linalg.norm(v)
    cth = v[2] / nv
    sth = np.sqrt(1 - cth ** 2)
    cph, sph = (1.0, 0.0) if sth == 0 else (v[0] / nv / sth, v[1] / nv / sth)
    T = np.array([[cph * cth, -sph * cth, -sth], [-sph, cph, 0.0], [cph * sth, sph * sth, cth]])
    return np.array([sch * ceta, sch * seta, cch]) @ T


def test_scattering_kinematics(orc):
    rng = np.random.default_rng(5)
    for _ in range(50):
        v = rng.normal(size=3)
        u1, u2 = rng.uniform(size=2)
        chi, eta = 2 * np.pi * u1, 2 * np.pi * u2
        d = orc.isotropic_scattering(v, u1, u2)
        assert np.allclose(d, _literal_rotation(v, np.sin(chi), np.cos(chi), np.sin(eta), np.cos(eta)), atol=1e-14)
        sch = np.sqrt(u1)
        r = orc.diffuse_reflection(v, u1, u2)
        assert np.allclose(r, _literal_rotation(v, sch, -np.sqrt(1 - sch ** 2), np.sin(eta), np.cos(eta)), atol=1e-14)
    # unrotated() is not orthogonal (row1.row2 = -2 sinϕ cosϕ cosθ): |v| is only
    # kept when ϕ = 0, e.g. v in the x-z half plane x >= 0
    d = orc.isotropic_scattering(np.array([1.0, 1.0, 1.0]), 0.3, 0.7)
    assert abs(np.linalg.norm(d) - 1) > 1e-3
    d = orc.isotropic_scattering(np.array([0.6, 0.0, 0.8]), 0.3, 0.7)
    assert abs(np.linalg.norm(d) - 1) < 1e-14
    # v along +z: the rotation is the identity (mcc.jl:98-101)
    d = orc.isotropic_scattering(np.array([0, 0, 2.0]), 0.125, 0.25)
    chi, eta = 2 * np.pi * 0.125, 2 * np.pi * 0.25
    assert np.allclose(d, [np.sin(chi) * np.cos(eta), np.sin(chi) * np.sin(eta), np.cos(chi)], atol=1e-15)


def test_mcc_max_sigma_g_constant_table(orc):
    eps = np.array([0.1, 10.0, 100.0])
    m = orc.mcc_max_sigma_g([(eps, np.full(3, 2e-19))], ME)
    assert abs(m - 2e-19 * np.sqrt(2 * 100.0 / orc.mass_ev(ME))) < 1e-12 * m


def test_golden_fixtures_reproduce():
    from tests.golden.make_golden import fixtures
    ref = np.load(os.path.join(HERE, "golden", "oracle_fixtures.npz"))
    new = fixtures()
    assert set(ref.files) == set(new)
    for k in ref.files:
        assert np.array_equal(ref[k], new[k]), k
