"""GPU parity tests: libiskra_gpu.so (through its C ABI) against the FP64 oracle.

Tolerances (stated by the north-star of this path):
  positions  |x_gpu - x_ref| <= 1e-6 * max(|x_ref|, Δx)          per particle
  velocities |v_gpu - v_ref| <= 1e-6 * max(|v_ref|, |v_in|)       per particle (3-vector norms)
  node charge max|ρ_gpu - ρ_ref| <= 1e-9 * max|ρ_ref|            on identical particle arrays
  potential  max|ϕ_gpu - ϕ_ref| <= 1e-7 * max|ϕ_ref| after solving to relative residual 1e-10
Push/gather run in FP32 on FP32 state, so each stage is compared from identical
inputs: the oracle receives the device's own (downloaded) state.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QE = 1.602176634e-19
ME = 9.1093837015e-31
MP = 1.67262192369e-27
EPS0 = 8.8541878128e-12


@pytest.fixture(scope="module")
def lib():
    from iskra_gb300 import _lib
    return _lib


def make_ctx(nx, ny, dx, dy, bcs=(0, 0, 0, 0)):
    from iskra_gb300.device import Context
    return Context(nx, ny, dx, dy, bcs)


def by_id(x, v, ids):
    o = np.argsort(ids)
    return np.asfortranarray(x[o]), np.asfortranarray(v[o]), ids[o]


def rand_particles(rng, n, nx, ny, dx, dy, vs):
    x = np.column_stack([rng.uniform(0, (nx - 1) * dx, n), rng.uniform(0, (ny - 1) * dy, n)])
    v = rng.normal(0, vs, (n, 3))
    return np.asfortranarray(x), np.asfortranarray(v)


def check_push(x_gpu, v_gpu, x_ref, v_ref, v_in, dx):
    ex = np.abs(x_gpu - x_ref).max(axis=1)
    sx = np.maximum(np.abs(x_ref).max(axis=1), dx)
    assert np.all(ex <= 1e-6 * sx), f"position error {np.max(ex / sx):.3e}"
    ev = np.linalg.norm(v_gpu - v_ref, axis=1)
    sv = np.maximum(np.linalg.norm(v_ref, axis=1), np.linalg.norm(v_in, axis=1))
    assert np.all(ev <= 1e-6 * sv + 1e-30), f"velocity error {np.max(ev / sv):.3e}"


@pytest.mark.parametrize("nx,ny,modes", [(65, 33, "wrap"), (129, 2, "wrap"), (40, 24, "discard_x")])
def test_advance_matches_oracle(orc, lib, nx, ny, modes):
    dx = dy = 1e-4
    rng = np.random.default_rng(nx * 7 + ny)
    n = 20000
    ctx = make_ctx(nx, ny, dx, dy)
    sid = ctx.species_create(-QE, ME, 1e3, n)
    if modes == "wrap":
        ctx.set_boundary(sid, lib.BND_WRAP, lib.BND_WRAP)
    else:
        ctx.set_boundary(sid, lib.BND_DISCARD, lib.BND_WRAP)
    x, v = rand_particles(rng, n, nx, ny, dx, dy, 3e5)
    ctx.upload(sid, x, v)
    E = np.asfortranarray(rng.normal(0, 2e3, (nx, ny, 3)))
    E[:, :, 2] = 0.0
    ctx.upload_E(E)
    x0, v0, i0 = by_id(*ctx.download(sid))  # the device's own (quantised) state
    dt = 1e-10
    ctx.advance(sid, dt)
    x1, v1, i1 = by_id(*ctx.download(sid))
    # oracle: gather + Boris + after_push on the same state, E read back as FP32
    E32 = E.astype(np.float32).astype(np.float64)
    xr, vr = x0.copy(order="F"), v0.copy(order="F")
    pu = orc.grid_to_particle(E32, dx, dy, xr)
    orc.push_cartesian(xr, vr, pu, None, -QE / ME, dt)
    wg = np.full(len(xr), 1e3)
    ids = i0.copy()
    if modes == "wrap":
        orc.wrap(xr, 0, nx, dx)
        orc.wrap(xr, 1, ny, dy)
        npn = len(xr)
        lo = hi = 0
    else:
        npn, lo, hi = orc.discard(xr, vr, wg, ids, 1e3, 0, nx, dx)
        xr, vr, ids = np.asfortranarray(xr[:npn]), np.asfortranarray(vr[:npn]), ids[:npn].copy()
        orc.wrap(xr, 1, ny, dy)
    o = np.argsort(ids)
    xr, vr, ids = xr[o], vr[o], ids[o]
    assert np.array_equal(ids, i1), "surviving particle set differs"
    vin = v0[np.searchsorted(i0, ids)]
    check_push(x1, v1, xr, vr, vin, dx)
    if modes != "wrap":
        ab = ctx.absorbed(sid)
        assert ab[0] == lo and ab[1] == hi and ab[2] == 0 and ab[3] == 0
    ctx.close()


# (9, 5): ~1600 particles per cell, past the 256 a window cell sums in
# one-word moments, so most runs take the two-word sums
@pytest.mark.parametrize("nx,ny", [(64, 64), (257, 2), (33, 17), (9, 5)])
def test_deposit_matches_oracle_and_is_order_independent(orc, lib, nx, ny):
    dx, dy = 2e-4, 1e-4
    rng = np.random.default_rng(nx + ny)
    n = 50000
    ctx = make_ctx(nx, ny, dx, dy, (0, 0, 1, 1))
    sid = ctx.species_create(QE, 40 * MP, 2.5e4, n)
    x, v = rand_particles(rng, n, nx, ny, dx, dy, 1e3)
    # corner cases: exactly on nodes and at the last representable offset
    x[0] = [0.0, 0.0]
    x[1] = [(nx - 1) * dx * (1 - 1e-12), (ny - 1) * dy * (1 - 1e-12)]
    x[2] = [3 * dx, (ny - 2) * dy]
    ctx.upload(sid, x, v)
    n_gpu = ctx.density(sid)
    xq, _, _ = ctx.download(sid)
    n_ref = orc.density(nx, ny, dx, dy, xq, 2.5e4, (0, 0, 1, 1))
    assert np.max(np.abs(n_gpu - n_ref)) <= 1e-9 * np.max(np.abs(n_ref))
    # total charge is conserved exactly up to the final FP64 conversion
    V = orc.cell_volume(nx, ny, dx, dy, (0, 0, 1, 1))
    assert abs(np.sum(n_gpu * V) - n * 2.5e4) <= 1e-12 * n * 2.5e4
    # bit-identical for a shuffled particle order
    perm = rng.permutation(len(xq))
    ctx2 = make_ctx(nx, ny, dx, dy, (0, 0, 1, 1))
    sid2 = ctx2.species_create(QE, 40 * MP, 2.5e4, n)
    ctx2.upload(sid2, xq[perm], np.zeros((len(xq), 3)))
    n2 = ctx2.density(sid2)
    assert np.array_equal(n2, n_gpu)
    ctx.close()
    ctx2.close()


def _setup_bc(target, kind, nx, ny):
    """Applies the same boundary setup to a device context or a PoissonOracle."""
    isdev = hasattr(target, "apply_periodic") and hasattr(target, "h")
    ap = target.apply_periodic
    ad = target.apply_dirichlet
    if kind == "slab":  # x Dirichlet columns (0 V, 100 V), y periodic (apply_periodic(solver, 1))
        ap(1)
        m1 = np.zeros((nx, ny), bool); m1[0, :] = True
        m2 = np.zeros((nx, ny), bool); m2[-1, :] = True
        ad(m1, 0.0)
        ad(m2, 100.0)
    elif kind == "periodic":  # apply_periodic(1) and (2): singular, mean-zero gauge
        ap(1)
        ap(2)
    elif kind == "neumann":  # floating electrode column i=1 (σ dof), grounded i=nx
        ap(1)
        dof = target.add_dof() if isdev else target.add_new_dof()
        m1 = np.zeros((nx, ny), bool); m1[0, :] = True
        m2 = np.zeros((nx, ny), bool); m2[-1, :] = True
        if isdev:
            target.apply_neumann(m1, dof)
            target.set_sigma(dof, 3.0e-6)
        else:
            target.apply_neumann(m1, dof)
            target.set_sigma(dof, 3.0e-6)
        ad(m2, 0.0)
    elif kind == "neumann_gauss":  # the same floating electrode with the Gauss-law rows (circuit runs)
        ap(1)
        dof = target.add_dof() if isdev else target.add_new_dof()
        m1 = np.zeros((nx, ny), bool); m1[0, :] = True
        m2 = np.zeros((nx, ny), bool); m2[-1, :] = True
        target.apply_neumann(m1, dof, gauss=True)
        target.set_sigma(dof, 3.0e-8)
        ad(m2, 0.0)
    elif kind == "open_box":  # no periodicity, a Dirichlet blob inside: CG path
        m1 = np.zeros((nx, ny), bool); m1[nx // 3:nx // 3 + 3, ny // 2:ny // 2 + 2] = True
        ad(m1, -20.0)
        m2 = np.zeros((nx, ny), bool); m2[:, 0] = True
        ad(m2, 0.0)


@pytest.mark.parametrize("kind,nx,ny", [("slab", 64, 64), ("slab", 130, 128), ("periodic", 128, 2),
                                        ("neumann", 257, 2), ("neumann", 33, 16), ("neumann_gauss", 257, 2),
                                        ("neumann_gauss", 64, 32), ("open_box", 31, 23),
                                        ("periodic", 32, 32)])
def test_poisson_matches_oracle(orc, lib, kind, nx, ny):
    dx = dy = 1e-3
    rng = np.random.default_rng(11)
    rho = rng.normal(0, 1e-6, (nx, ny))
    if kind == "periodic":
        rho -= rho.mean()
    ctx = make_ctx(nx, ny, dx, dy)
    ctx.poisson_create(EPS0)
    _setup_bc(ctx, kind, nx, ny)
    ps = orc.PoissonOracle(nx, ny, dx, dy, EPS0)
    _setup_bc(ps, kind, nx, ny)
    rtol = 1e-11 if kind == "open_box" else 1e-10  # direct FFT/tridiagonal solves: FP64 floor ~1e-11
    phi_g, it, rr = ctx.solve_host(-rho, rtol=rtol, maxit=20000)
    assert rr <= rtol
    phi_o = ps.solve(-rho)
    if kind == "periodic":
        phi_o = phi_o - phi_o.mean()
    scale = np.max(np.abs(phi_o))
    assert np.max(np.abs(phi_g - phi_o)) <= 1e-7 * scale, f"{kind}: {np.max(np.abs(phi_g - phi_o)) / scale:.2e}"
    E_g = ctx.field(lib.FIELD_E)
    E_o = orc.electric_field(phi_o, dx, dy)
    assert np.max(np.abs(E_g - E_o)) <= 1e-6 * np.max(np.abs(E_o))
    sep = ctx.set_method(0)
    if kind in ("slab", "periodic", "neumann", "neumann_gauss") and (ny & (ny - 1)) == 0:
        assert sep == 0, "separable operator expected to use the FFT/tridiagonal solve"
    ctx.close()


def test_parallel_capacitor_kat(lib):
    """FiniteDifferenceMethod/test/runtests.jl:8-22: 3x5 nodes at 0.5 m spacing,
    0 V at column 1, 1 V at column 3 -> E_x = -1, E_y = 0."""
    ctx = make_ctx(3, 5, 0.5, 0.5)
    ctx.poisson_create(EPS0)
    m1 = np.zeros((3, 5), bool); m1[0, :] = True
    m2 = np.zeros((3, 5), bool); m2[2, :] = True
    ctx.apply_dirichlet(m1, 0.0)
    ctx.apply_dirichlet(m2, 1.0)
    ctx.solve_host(np.zeros((3, 5)), rtol=1e-14, maxit=1000)
    E = ctx.field(lib.FIELD_E)
    assert np.allclose(E[:, :, 0], -1.0, rtol=0, atol=1e-12)
    assert np.linalg.norm(E[:, :, 1]) <= 1e-15
    ctx.close()


def test_circuit_step_matches_oracle(orc, lib):
    nx, ny, dx = 65, 2, 0.025 / 64
    ctx = make_ctx(nx, ny, dx, dx)
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    dof = ctx.add_dof()
    m1 = np.zeros((nx, ny), bool); m1[0, :] = True
    m2 = np.zeros((nx, ny), bool); m2[-1, :] = True
    ctx.apply_neumann(m1, dof)
    ctx.apply_dirichlet(m2, 0.0)
    area = dx * 1.0
    R, L, C, amp, f = 50.0, 1e-6, 1e-9, 300.0, 13.56e6
    ctx.circuit_create(R, L, C, amp, f, 0.0, dof, m1, m2, area, 1.0)
    rho = np.zeros((nx, ny))
    state = np.zeros(3)
    sigma = 0.0
    dt = 7.4e-11
    for n in range(5):
        phi, _, _ = ctx.solve_host(-rho, rtol=1e-10)
        vext = phi[0, 0] - phi[-1, 0]
        ctx.circuit_advance(dt)
        st = ctx.circuit_state()
        state = orc.advance_circuit(R, L, C, state, vext, amp * np.sin(2 * np.pi * f * state[2]), dt)
        sigma += -dt * state[0] / area
        assert abs(st["i"] - state[0]) <= 1e-12 * max(abs(state[0]), 1e-30)
        assert abs(st["q"] - state[1]) <= 1e-12 * max(abs(state[1]), 1e-30)
        assert abs(st["sigma"] - sigma) <= 1e-12 * max(abs(sigma), 1e-30)
    ctx.close()


def _argon_tables(ne=1024):
    eps = np.logspace(-2, 3, ne)
    el = np.full(ne, 1e-19)
    ex = np.where(eps > 11.5, np.minimum((eps - 11.5) / (100 - 11.5), 1.0) * 3e-21, 0.0)
    iz = np.where(eps > 15.76, 3e-20 * np.log(eps / 15.76) / np.log(100 / 15.76) * (100 / eps) ** 0.5, 0.0)
    return eps, el, ex, iz


@pytest.mark.parametrize("table", ["log-uniform", "non-uniform"])
def test_mcc_counts_statistics(orc, lib, table):
    """Constant-σ elastic + excitation/ionisation on a uniform gas: accepted
    counts per process against the oracle's reference algorithm (3σ).
    "non-uniform": the same cross sections on linearly spaced energies, 2600
    per process (7800 table nodes: bisection lookups on tables staged in
    62 KB of shared memory, above the 48 KB a launch gets without opting in)."""
    nx, ny, dx = 33, 2, 1e-3
    n = 100000
    rng = np.random.default_rng(5)
    x, _ = rand_particles(rng, n, nx, ny, dx, dx, 1.0)
    speed = np.sqrt(2 * 40.0 * QE / ME)  # 40 eV electrons, isotropic
    d = rng.normal(size=(n, 3))
    v = np.asfortranarray(speed * d / np.linalg.norm(d, axis=1)[:, None])
    eps, el, ex, iz = _argon_tables()
    if table == "non-uniform":
        lin = np.linspace(0.01, 1000.0, 2600)
        el, ex, iz = (np.interp(lin, eps, t) for t in (el, ex, iz))
        eps = lin
    procs_dev = [(lib.MCC_ELASTIC_ISOTROPIC, 0.0, eps, el), (lib.MCC_EXCITATION, 11.5, eps, ex),
                 (lib.MCC_IONIZATION, 15.76, eps, iz)]
    gas_n = np.full((nx, ny), 7.24e20)
    dt = 7.4e-11
    ctx = make_ctx(nx, ny, dx, dx)
    se = ctx.species_create(-QE, ME, 1.0, 2 * n)
    si = ctx.species_create(QE, 40 * MP, 1.0, 2 * n)
    ctx.upload(se, x, v)
    mid, msg = ctx.mcc_create(se, procs_dev, 40 * MP, 300.0, gas_n, product=si)
    steps = 20
    for s in range(steps):
        ctx.mcc_perform(mid, dt, 99, s + 1)
    cg = np.array(ctx.mcc_counts(mid, 3), float)
    ne_dev = ctx.count(se)
    ni_dev = ctx.count(si)
    # oracle (reference algorithm, own RNG)
    procs_o = [("elastic_isotropic", 0.0, eps, el), ("excitation", 11.5, eps, ex), ("ionization", 15.76, eps, iz)]
    m = orc.MCCOracle(procs_o, ME, -QE, 1.0, 40 * MP, 300.0, product_w0=1.0)
    assert abs(m.max_sigma_g - msg) <= 1e-12 * msg
    cap = 2 * n
    sx = np.zeros((cap, 2), order="F"); sx[:n] = x
    sv = np.zeros((cap, 3), order="F"); sv[:n] = v
    px = np.zeros((cap, 2), order="F"); pv = np.zeros((cap, 3), order="F")
    E = np.zeros((nx, ny, 3), order="F")
    snp, pnp = n, 0
    co = np.zeros(3)
    for s in range(steps):
        snp, pnp, c = m.perform(E, gas_n, dx, dx, dt, sx, sv, snp, 1234 + s, px, pv, pnp)
        co += c
    for k in range(3):
        sd = np.sqrt(cg[k] + co[k]) + 1.0
        assert abs(cg[k] - co[k]) <= 3 * sd, f"process {k}: gpu {cg[k]} oracle {co[k]}"
    # ionisation conserves pairs: one electron and one ion per ionisation event
    assert ne_dev - n == ni_dev
    assert abs(ni_dev - cg[2]) <= 0.01 * cg[2] + 2  # second ionisation of one particle in one step adds no child
    ctx.close()


def test_elastic_scattering_heavy_target_keeps_speed_for_phi0(lib):
    """Elastic scattering off an infinitely heavy, cold target.  The reference's
    unrotated() (mcc.jl:83-87) is orthogonal only for ϕ = 0, so |v| is kept
    for velocities in the x-z half plane x >= 0 and changes otherwise."""
    nx, ny, dx = 17, 2, 1e-3
    n = 50000
    rng = np.random.default_rng(9)
    x, _ = rand_particles(rng, n, nx, ny, dx, dx, 1.0)
    th = rng.uniform(0.05, np.pi - 0.05, n)
    v = np.asfortranarray(np.column_stack([1e6 * np.sin(th), np.zeros(n), 1e6 * np.cos(th)]))
    eps = np.array([0.01, 1000.0])
    ctx = make_ctx(nx, ny, dx, dx)
    se = ctx.species_create(-QE, ME, 1.0, n)
    ctx.upload(se, x, v)
    mid, _ = ctx.mcc_create(se, [(lib.MCC_ELASTIC_ISOTROPIC, 0.0, eps, [1e-19, 1e-19])], 1e10, 0.0,
                            np.full((nx, ny), 1e21))
    ctx.mcc_perform(mid, 1e-10, 3, 1)
    c = ctx.mcc_counts(mid, 1)
    assert c[0] > 100
    _, v1, _ = ctx.download(se)
    sp = np.linalg.norm(v1, axis=1)
    ok = np.abs(sp - 1e6) <= 2e-6 * 1e6
    moved = np.abs(v1[:, 1]) > 1.0  # scattered particles left the y = 0 plane
    assert moved.sum() >= 0.9 * c[0]
    # a particle selected twice in the step scatters the second time with ϕ ≠ 0
    # (non-orthogonal frame): only those few may change speed
    assert np.sum(~ok) <= max(3, 0.05 * c[0])
    ctx.close()


def test_full_step_matches_oracle_two_species(orc, lib):
    """One iskra_step (advance both species -> ρ -> Poisson -> E) on a slab
    with discard in x, wrap in y, against the oracle run on the same state."""
    nx, ny, dx = 64, 32, 1e-4
    n = 30000
    rng = np.random.default_rng(21)
    ctx = make_ctx(nx, ny, dx, dx, (0, 0, 1, 1))
    se = ctx.species_create(-QE, ME, 2e4, n)
    si = ctx.species_create(QE, 40 * MP, 2e4, n)
    for s in (se, si):
        ctx.set_boundary(s, lib.BND_DISCARD, lib.BND_WRAP)
    xe, ve = rand_particles(rng, n, nx, ny, dx, dx, 8e5)
    xi, vi = rand_particles(rng, n, nx, ny, dx, dx, 3e2)
    ctx.upload(se, xe, ve)
    ctx.upload(si, xi, vi)
    ctx.poisson_create(EPS0)
    _setup_bc(ctx, "slab", nx, ny)
    ctx.step(1e-11, 1, seed=0, rtol=1e-10)   # E = 0 -> free push, deposit, solve
    ctx.sync()
    state = [by_id(*ctx.download(s)) for s in (se, si)]
    E1 = ctx.field(lib.FIELD_E)
    rho = ctx.field(lib.FIELD_RHO)
    ps = orc.PoissonOracle(nx, ny, dx, dx, EPS0)
    _setup_bc(ps, "slab", nx, ny)
    rho_o = sum(q * orc.density(nx, ny, dx, dx, st[0], 2e4, (0, 0, 1, 1)) for q, st in ((-QE, state[0]), (QE, state[1])))
    assert np.max(np.abs(rho - rho_o)) <= 1e-9 * np.max(np.abs(rho_o))
    phi_o = ps.solve(-rho_o)
    E_o = orc.electric_field(phi_o, dx, dx)
    assert np.max(np.abs(E1 - E_o)) <= 1e-6 * np.max(np.abs(E_o))
    # second step uses this E: compare the push of species 0
    x0, v0, i0 = state[0]
    ctx.step(1e-11, 1, seed=0, rtol=1e-10)
    ctx.sync()
    x1, v1, i1 = by_id(*ctx.download(se))
    E32 = E1.copy(order="F")
    E32[:, :, :2] = E1[:, :, :2].astype(np.float32)
    xr, vr = x0.copy(order="F"), v0.copy(order="F")
    pu = orc.grid_to_particle(E32, dx, dx, xr)
    orc.push_cartesian(xr, vr, pu, None, -QE / ME, 1e-11)
    wg = np.full(len(xr), 2e4)
    ids = i0.copy()
    npn, _, _ = orc.discard(xr, vr, wg, ids, 2e4, 0, nx, dx)
    xr, vr, ids = np.asfortranarray(xr[:npn]), np.asfortranarray(vr[:npn]), ids[:npn].copy()
    orc.wrap(xr, 1, ny, dx)
    o = np.argsort(ids)
    assert np.array_equal(ids[o], i1)
    check_push(x1, v1, xr[o], vr[o], v0[np.searchsorted(i0, ids[o])], dx)
    ctx.close()


def test_errors_are_reported_not_trapped(lib):
    from iskra_gb300._lib import IskraError
    ctx = make_ctx(16, 16, 1e-3, 1e-3)
    sid = ctx.species_create(-QE, ME, 1.0, 10)
    with pytest.raises(IskraError) as e:
        ctx.upload(sid, np.zeros((11, 2)), np.zeros((11, 3)))
    assert e.value.code == 3  # ECAPACITY
    with pytest.raises(IskraError) as e:
        ctx.upload(sid, np.array([[1.0, 0.0]]), np.zeros((1, 3)))  # outside the grid
    assert e.value.code == 4  # EDOMAIN
    with pytest.raises(IskraError) as e:
        ctx.upload(sid, np.array([[5e-3, 5e-3]]), np.array([[np.nan, 0.0, 0.0]]))
    assert e.value.code == 6  # ENAN
    ctx.sync()  # the context stays usable
    ctx.close()


def test_cross_section_lookup_matches_oracle(orc, lib):
    """CrossSection (cross_section.jl:8-16) as the MCC kernels evaluate it
    (FP32 table, bracket by log-uniform guess or bisection) against the
    oracle's FP64 interpolation of the same FP32-rounded table at the same
    FP32-rounded energies: below the first node, on nodes, between nodes,
    above the last node; a log-uniform table (1024 nodes), a non-uniform
    table, a two-node and a one-node table.  |σ_gpu - σ_ref| <= 1e-6 max σ."""
    nx, ny, dx = 9, 2, 1e-3
    rng = np.random.default_rng(17)
    eps_lu = np.logspace(-2, 3, 1024)
    sig_lu = 3e-20 * (1 + np.sin(np.log(eps_lu)) ** 2)
    eps_nu = np.sort(rng.uniform(0.05, 500.0, 300))
    sig_nu = rng.uniform(1e-21, 5e-19, 300)
    tables = [(eps_lu, sig_lu), (eps_nu, sig_nu), (np.array([1.0, 20.0]), np.array([2e-20, 8e-20])),
              (np.array([5.0]), np.array([4e-20]))]
    ctx = make_ctx(nx, ny, dx, dx)
    se = ctx.species_create(-QE, ME, 1.0, 16)
    procs = [(lib.MCC_ELASTIC_ISOTROPIC, 0.0, e, s) for e, s in tables]
    mid, _ = ctx.mcc_create(se, procs, 40 * MP, 300.0, np.full((nx, ny), 1e20))
    for k, (e, s) in enumerate(tables):
        lo, hi = e[0], e[-1]
        probes = np.concatenate([[0.0, lo * 0.5, lo, hi, hi * 2.0, 1e4], e[:: max(1, len(e) // 50)],
                                 rng.uniform(lo, hi, 2000), np.exp(rng.uniform(np.log(lo), np.log(hi), 2000))])
        g = ctx.mcc_sigma(mid, k, probes)
        e32 = e.astype(np.float32).astype(np.float64)
        s32 = s.astype(np.float32).astype(np.float64)
        ref = np.array([orc.sigma(e32, s32, float(np.float32(x))) for x in probes])
        err = np.max(np.abs(g - ref))
        assert err <= 1e-6 * np.max(s), f"table {k}: max |σ_gpu - σ_ref| {err:.3e} (max σ {np.max(s):.3e})"
        # flat extrapolation outside the table (cross_section.jl:13)
        assert g[0] == s32[0] and g[1] == s32[0] and g[4] == s32[-1] and g[5] == s32[-1]
    ctx.close()
