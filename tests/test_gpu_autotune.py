"""Sort cadence and push tile size: results do not depend on them, and the
autotuners pick them.

The sort only permutes the particle store; push and boundary rules act per
particle, the deposit sums integers (order-independent), so two runs from the
same particles with very different sort periods must agree bit for bit (ρ,
every particle by id, wall-absorbed counts).  iskra_autotune_sort then times
the speed-based periods scaled by 0.5, 1, 2 and 4 on the run itself and keeps
one of them."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QE, ME, MAR, EPS0 = 1.602176634e-19, 9.1093837015e-31, 6.6335209e-26, 8.8541878128e-12
N, NP, DX, DT = 128, 300000, 1e-4, 1e-11


def _slab(lib, sort_every):
    from iskra_gb300.device import Context
    rng = np.random.default_rng(9)
    L = (N - 1) * DX
    ctx = Context(N, N, DX, DX, (0, 0, 0, 0))
    sids = []
    for q, m, T in ((-QE, ME, 2.0), (QE, MAR, 0.03)):
        s = ctx.species_create(q, m, 1e15 * L * L / NP, NP)
        ctx.set_boundary(s, lib.BND_DISCARD, lib.BND_WRAP)
        x = np.asfortranarray(np.column_stack([rng.uniform(0, L, NP), rng.uniform(0, L, NP)]))
        v = np.asfortranarray(rng.standard_normal((NP, 3)) * np.sqrt(T * QE / m))
        ctx.upload(s, x, v)
        sids.append(s)
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    left = np.zeros((N, N), bool)
    left[0, :] = True
    right = np.zeros((N, N), bool)
    right[-1, :] = True
    ctx.apply_dirichlet(left, 0.0)
    ctx.apply_dirichlet(right, 100.0)
    ctx.set_sort_every(sort_every)
    return ctx, sids


def test_results_do_not_depend_on_sort_cadence(lib):
    a, sa = _slab(lib, 3)
    b, sb = _slab(lib, 40)
    a.step(DT, 40, seed=1, rtol=1e-8)
    b.step(DT, 40, seed=1, rtol=1e-8)
    assert np.array_equal(a.field(lib.FIELD_RHO), b.field(lib.FIELD_RHO))
    for s in (0, 1):
        xa, va, ia = a.download(sa[s])
        xb, vb, ib = b.download(sb[s])
        oa, ob = np.argsort(ia), np.argsort(ib)
        assert np.array_equal(ia[oa], ib[ob])
        assert np.array_equal(xa[oa], xb[ob]) and np.array_equal(va[oa], vb[ob])
        assert a.absorbed(sa[s]) == b.absorbed(sb[s])
    a.close()
    b.close()


def test_autotune_sort_picks_a_factor(lib):
    ctx, _ = _slab(lib, -1)
    f, ms = ctx.autotune_sort(DT, trial=16, seed=1)
    assert f in (0.5, 1.0, 2.0, 4.0) and ms > 0
    ctx.step(DT, 10, seed=1, rtol=1e-8)
    ctx.sync()
    assert ctx.solve_info()[1] <= 1e-8
    ctx.set_sort_every(5)
    with pytest.raises(Exception):
        ctx.autotune_sort(DT, trial=4)
    ctx.close()


@pytest.mark.parametrize("cells", [8, 32])
def test_results_do_not_depend_on_tile_size(lib, cells):
    """The push tile (8, 16 or 32 cells per axis) only decides which block
    pushes a particle: runs with different tiles agree bit for bit."""
    a, sa = _slab(lib, -1)
    b, sb = _slab(lib, -1)
    assert a.tile() == 16
    b.set_tile(cells)
    assert b.tile() == cells
    a.step(DT, 40, seed=1, rtol=1e-8)
    b.step(DT, 20, seed=1, rtol=1e-8)
    b.set_tile(16 if cells == 32 else 32)  # a change in the middle of a run
    b.step(DT, 20, seed=1, rtol=1e-8)
    assert np.array_equal(a.field(lib.FIELD_RHO), b.field(lib.FIELD_RHO))
    assert np.array_equal(a.field(lib.FIELD_PHI), b.field(lib.FIELD_PHI))
    for s in (0, 1):
        xa, va, ia = a.download(sa[s])
        xb, vb, ib = b.download(sb[s])
        oa, ob = np.argsort(ia), np.argsort(ib)
        assert np.array_equal(ia[oa], ib[ob])
        assert np.array_equal(xa[oa], xb[ob]) and np.array_equal(va[oa], vb[ob])
        assert a.absorbed(sa[s]) == b.absorbed(sb[s])
    with pytest.raises(Exception):
        b.set_tile(12)
    a.close()
    b.close()


def test_autotune_picks_tile_and_cadence(lib):
    """iskra_autotune times every (tile, sort factor) pair on the run and keeps
    the fastest; a second context of the same shape takes the cached choice."""
    ctx, _ = _slab(lib, -1)
    tile, f, ms, grid, cached = ctx.autotune(DT, trial=8, seed=1)
    assert not cached and tile in (8, 16, 32) and f in (0.5, 1.0, 2.0, 4.0)
    assert len(grid) == 12 and all(v > 0 for v in grid.values())
    assert ms == min(grid.values()) and grid[(tile, f)] == ms
    assert ctx.tile() == tile
    print("autotune (tile, sort factor) -> ms per step:", {k: round(v, 4) for k, v in grid.items()})
    ctx.step(DT, 5, seed=1, rtol=1e-8)
    assert ctx.solve_info()[1] <= 1e-8
    other, _ = _slab(lib, -1)
    t2, f2, ms2, grid2, cached2 = other.autotune(DT, trial=8, seed=1)
    assert cached2 and grid2 is None and (t2, f2, ms2) == (tile, f, ms) and other.tile() == tile
    ctx.close()
    other.close()


def test_double_float_rho_matches_fp64_rho(lib):
    """ρ and the densities formed in double-float (tolerance 1e-8: the
    separable solver's double-float state) equal the FP64 ones (tolerance
    1e-12) of the same deposit to ~2^-48 relative."""
    a, sa = _slab(lib, -1)
    b, sb = _slab(lib, -1)
    a.step(DT, 1, seed=1, rtol=1e-8)
    b.step(DT, 1, seed=1, rtol=1e-12)
    ra, rb = a.field(lib.FIELD_RHO), b.field(lib.FIELD_RHO)
    scale = np.max(np.abs(rb))
    assert scale > 0 and np.max(np.abs(ra - rb)) <= 1e-13 * scale
    for s in (0, 1):
        na, nb = a.density(sa[s]), b.density(sb[s])
        assert np.max(np.abs(na - nb)) <= 1e-13 * np.max(np.abs(nb))
    a.close()
    b.close()


def test_rho_download_between_steps_is_current(lib):
    """ρ read between iskra_step calls (each read makes the FP64 copy) is the
    ρ of the latest step: equal to a run that reads only at the end."""
    a, _ = _slab(lib, -1)
    b, _ = _slab(lib, -1)
    seen = []
    for _ in range(3):
        a.step(DT, 1, seed=1, rtol=1e-8)
        seen.append(a.field(lib.FIELD_RHO))
    b.step(DT, 3, seed=1, rtol=1e-8)
    assert not np.array_equal(seen[0], seen[2])
    assert np.array_equal(seen[2], b.field(lib.FIELD_RHO))
    a.close()
    b.close()


def test_species_pair_push_matches_single_species_pushes(lib):
    """The step's two-species push launch and one push launch per species
    (iskra_advance) move every particle to the same bits in the same field."""
    rng = np.random.default_rng(12)
    E = np.asfortranarray(rng.standard_normal((N, N, 3)) * 2e4)
    E[:, :, 2] = 0.0
    a, sa = _slab(lib, -1)
    b, sb = _slab(lib, -1)
    a.upload_E(E)
    b.upload_E(E)
    a.step(DT, 1, seed=1, rtol=1e-8)          # the push reads the uploaded E
    for s in sb:
        b.advance(s, DT)
    for s in (0, 1):
        xa, va, ia = a.download(sa[s])
        xb, vb, ib = b.download(sb[s])
        oa, ob = np.argsort(ia), np.argsort(ib)
        assert np.array_equal(ia[oa], ib[ob])
        assert np.array_equal(xa[oa], xb[ob]) and np.array_equal(va[oa], vb[ob])
    a.close()
    b.close()
