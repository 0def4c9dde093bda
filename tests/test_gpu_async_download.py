"""Non-blocking field download (iskra_field_download_async): ϕ of each step,
copied to host buffers while later steps run, equals the blocking download of
the same step bit for bit once a synchronising call has returned."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QE, ME, MAR, EPS0 = 1.602176634e-19, 9.1093837015e-31, 6.6335209e-26, 8.8541878128e-12


def test_async_phi_matches_blocking_download(lib):
    from iskra_gb300.device import Context
    n, npart, dx = 64, 100000, 1e-4
    L = (n - 1) * dx

    def make():
        ctx = Context(n, n, dx, dx, (0, 0, 0, 0))
        r = np.random.default_rng(3)
        for q, m, T in ((-QE, ME, 2.0), (QE, MAR, 0.03)):
            s = ctx.species_create(q, m, 1e15 * L * L / npart, npart)
            ctx.set_boundary(s, lib.BND_DISCARD, lib.BND_WRAP)
            x = np.asfortranarray(np.column_stack([r.uniform(0, L, npart), r.uniform(0, L, npart)]))
            v = np.asfortranarray(r.standard_normal((npart, 3)) * np.sqrt(T * QE / m))
            ctx.upload(s, x, v)
        ctx.poisson_create(EPS0)
        ctx.apply_periodic(1)
        left = np.zeros((n, n), bool)
        left[0, :] = True
        right = np.zeros((n, n), bool)
        right[-1, :] = True
        ctx.apply_dirichlet(left, 0.0)
        ctx.apply_dirichlet(right, 100.0)
        return ctx

    a, b = make(), make()
    outs = [np.zeros((n, n), order="F") for _ in range(5)]
    ref = []
    for k in range(5):
        a.step(1e-11, 1, seed=1, rtol=1e-8)
        a.field_async(lib.FIELD_PHI, outs[k])
        b.step(1e-11, 1, seed=1, rtol=1e-8)
        ref.append(b.field(lib.FIELD_PHI))
    a.sync()
    for k in range(5):
        assert np.array_equal(outs[k], ref[k]), k
    # E and ρ through the same path
    e = np.zeros((n, n, 3), order="F")
    a.field_async(lib.FIELD_E, e)
    a.sync()
    assert np.array_equal(e, b.field(lib.FIELD_E))
    a.close()
    b.close()
