"""Multigrid-preconditioned CG (the solver of non-separable operators) against
the oracle's LU of the reference's assembled operator: an internal Dirichlet
electrode, open or y-periodic boundaries, a floating electrode (σ dof) that
is not a whole column.  Tolerances as tests/test_gpu_parity.py: ϕ within 1e-7
of max|ϕ| and E within 1e-6 of max|E| after a solve to relative residual
1e-10.  The multigrid cycle must keep the iteration count small (the
Jacobi-scaled CG it replaces needs hundreds to thousands at these sizes)."""
import numpy as np
import pytest

from test_gpu_parity import EPS0, make_ctx

pytestmark = pytest.mark.gpu


def _setup(target, kind, nx, ny, isdev):
    ad = target.apply_dirichlet
    blob = np.zeros((nx, ny), bool)
    blob[nx // 3:nx // 3 + 5, ny // 2:ny // 2 + 4] = True
    bottom = np.zeros((nx, ny), bool)
    bottom[:, 0] = True
    if kind == "open":
        ad(blob, -20.0)
        ad(bottom, 0.0)
    elif kind == "periodic_y":
        target.apply_periodic(1)
        ad(blob, 35.0)
        left = np.zeros((nx, ny), bool)
        left[0, :] = True
        ad(left, 0.0)
    elif kind == "floating":  # a floating electrode column, an internal electrode, a grounded wall
        target.apply_periodic(1)
        dof = target.add_dof() if isdev else target.add_new_dof()
        plate = np.zeros((nx, ny), bool)
        plate[0, :] = True
        target.apply_neumann(plate, dof, gauss=True)
        target.set_sigma(dof, 2.0e-8)
        right = np.zeros((nx, ny), bool)
        right[-1, :] = True
        ad(right, 0.0)
        ad(blob, 10.0)


@pytest.mark.parametrize("kind,nx,ny", [("open", 200, 160), ("periodic_y", 257, 128), ("floating", 130, 96),
                                        ("open", 31, 23)])
def test_multigrid_cg_matches_oracle(orc, lib, kind, nx, ny):
    dx = 1e-3
    rng = np.random.default_rng(5)
    rho = rng.normal(0, 1e-6, (nx, ny))
    ctx = make_ctx(nx, ny, dx, dx)
    ctx.poisson_create(EPS0)
    _setup(ctx, kind, nx, ny, True)
    assert ctx.set_method(0) == 2, "non-separable operator expected to use multigrid CG"
    phi_g, it, rr = ctx.solve_host(-rho, rtol=1e-10, maxit=500)
    assert rr <= 1e-10
    assert it <= 40, f"{kind}: {it} multigrid-CG iterations"
    ps = orc.PoissonOracle(nx, ny, dx, dx, EPS0)
    _setup(ps, kind, nx, ny, False)
    phi_o = ps.solve(-rho)
    scale = np.max(np.abs(phi_o))
    assert np.max(np.abs(phi_g - phi_o)) <= 1e-7 * scale, f"{kind}: {np.max(np.abs(phi_g - phi_o)) / scale:.2e}"
    E_g = ctx.field(lib.FIELD_E)
    E_o = orc.electric_field(phi_o, dx, dx)
    assert np.max(np.abs(E_g - E_o)) <= 1e-6 * np.max(np.abs(E_o))
    ctx.close()
    # the Jacobi-scaled CG, from the same zero start, reaches the same solution
    # with many more iterations
    ctx = make_ctx(nx, ny, dx, dx)
    ctx.poisson_create(EPS0)
    _setup(ctx, kind, nx, ny, True)
    assert ctx.set_method(1) == 1
    phi_j, it_j, rr_j = ctx.solve_host(-rho, rtol=1e-10, maxit=20000)
    print(f"{kind} {nx}x{ny}: multigrid CG {it} iterations, Jacobi CG {it_j}")
    assert rr_j <= 1e-10 and it_j > 3 * it
    assert np.max(np.abs(phi_j - phi_o)) <= 1e-7 * scale
    ctx.close()


def test_multigrid_cg_on_a_separable_operator_matches_the_direct_solve(lib):
    """method 2 forces multigrid CG on the slab the FFT/tridiagonal solve takes:
    both meet the same residual, so their potentials agree to the tolerance."""
    nx, ny, dx = 130, 64, 1e-4
    rng = np.random.default_rng(8)
    rho = rng.normal(0, 1e-5, (nx, ny))
    out = {}
    for method in (0, 2):
        ctx = make_ctx(nx, ny, dx, dx)
        ctx.poisson_create(EPS0)
        ctx.apply_periodic(1)
        left = np.zeros((nx, ny), bool)
        left[0, :] = True
        right = np.zeros((nx, ny), bool)
        right[-1, :] = True
        ctx.apply_dirichlet(left, 0.0)
        ctx.apply_dirichlet(right, 100.0)
        assert ctx.set_method(method) == method
        out[method] = ctx.solve_host(-rho, rtol=1e-11, maxit=500)
        ctx.close()
    phi0, phi2 = out[0][0], out[2][0]
    assert out[2][2] <= 1e-11
    assert np.max(np.abs(phi0 - phi2)) <= 1e-8 * np.max(np.abs(phi0))


def test_multigrid_cg_inside_steps(lib):
    """A slab with an internal electrode stepped with particles: every step's
    solve meets the tolerance through multigrid CG (eager step path)."""
    from test_gpu_parity import ME, QE, rand_particles
    nx, ny, dx = 96, 64, 1e-4
    ctx = make_ctx(nx, ny, dx, dx)
    rng = np.random.default_rng(3)
    se = ctx.species_create(-QE, ME, 5e4, 40000)
    ctx.set_boundary(se, lib.BND_DISCARD, lib.BND_WRAP)
    ctx.upload(se, *rand_particles(rng, 40000, nx, ny, dx, dx, 2e5))
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    left = np.zeros((nx, ny), bool)
    left[0, :] = True
    right = np.zeros((nx, ny), bool)
    right[-1, :] = True
    blob = np.zeros((nx, ny), bool)
    blob[40:46, 20:30] = True
    ctx.apply_dirichlet(left, 0.0)
    ctx.apply_dirichlet(right, 0.0)
    ctx.apply_dirichlet(blob, 50.0)
    assert ctx.set_method(0) == 2
    for _ in range(5):
        ctx.step(1e-11, 1, seed=1, rtol=1e-8)
        it, rr = ctx.solve_info()
        assert rr <= 1e-8 and it <= 30
    ctx.close()
