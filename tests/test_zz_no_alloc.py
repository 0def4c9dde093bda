"""iskra_density_noalloc: the density entry point that allocates no device
memory, for callers that cannot call cudaMalloc (a host framework that owns
all device memory, or code inside another library's stream capture).

It is checked through the C ABI against the allocating entry point
(iskra_density) on the same particles, within the node-charge tolerance of the
parity tests (1e-9 relative), on two calls in a row: the second call must not
see the first call's accumulator.  This file is collected last so that a run
stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QE = 1.602176634e-19


def test_density_noalloc_matches_density():
    torch = pytest.importorskip("torch")
    from iskra_gb300 import _lib
    from iskra_gb300.device import Context

    nx, ny, dx, dy = 96, 80, 1e-4, 2e-4
    bcs = (0, 0, 1, 1)
    rng = np.random.default_rng(123)
    lib = _lib.load()
    grid = _lib.Grid(nx, ny, dx, dy, 0.0, 0.0, (ctypes.c_int32 * 4)(*bcs))
    stream = torch.cuda.current_stream()
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    results = []
    for call, (n, w0) in enumerate(((40000, 3.0e4), (25000, 7.5e3))):
        ctx = Context(nx, ny, dx, dy, bcs)
        sid = ctx.species_create(QE, 6.6e-26, w0, n)
        x = np.column_stack([rng.uniform(0, (nx - 1) * dx, n), rng.uniform(0, (ny - 1) * dy, n)])
        ctx.upload(sid, x, np.zeros((n, 3)))
        n_ref = ctx.density(sid)                     # existing (allocating) entry point
        xq, _, _ = ctx.download(sid)                 # the device's own quantised positions
        ctx.close()
        x_dev = torch.from_numpy(np.ascontiguousarray(xq.T).reshape(-1)).to("cuda")  # column-major (n x 2)
        n_dev = torch.full((nx * ny,), -1.0, dtype=torch.float64, device="cuda")
        rc = lib.iskra_density_noalloc(ctypes.byref(grid), ctypes.c_void_p(x_dev.data_ptr()), n, n, w0,
                                       ctypes.c_void_p(n_dev.data_ptr()), ctypes.c_void_p(flag.data_ptr()),
                                       stream.cuda_stream)
        assert rc == 0
        torch.cuda.synchronize()
        assert int(flag.item()) == 0
        n_gpu = n_dev.cpu().numpy().reshape((nx, ny), order="F")
        assert np.max(np.abs(n_gpu - n_ref)) <= 1e-9 * np.max(np.abs(n_ref)), f"call {call}"
        results.append(n_gpu)
    assert not np.array_equal(results[0], results[1])


def test_density_noalloc_rejects_oversized_grid():
    from iskra_gb300 import _lib
    lib = _lib.load()
    grid = _lib.Grid(2048, 1024, 1e-4, 1e-4, 0.0, 0.0, (ctypes.c_int32 * 4)(0, 0, 0, 0))
    rc = lib.iskra_density_noalloc(ctypes.byref(grid), None, 0, 0, 1.0, ctypes.c_void_p(8), ctypes.c_void_p(8), 0)
    assert rc == 1  # ISKRA_EINVAL: the grid exceeds the static accumulator; nothing is launched


def test_density_noalloc_rejects_grid_origin():
    """particle_cell ignores the origin, so a grid with one is refused like iskra_ctx_create does."""
    from iskra_gb300 import _lib
    lib = _lib.load()
    grid = _lib.Grid(64, 64, 1e-4, 1e-4, 1e-3, 0.0, (ctypes.c_int32 * 4)(0, 0, 0, 0))
    rc = lib.iskra_density_noalloc(ctypes.byref(grid), None, 0, 0, 1.0, ctypes.c_void_p(8), ctypes.c_void_p(8), 0)
    assert rc == 1  # ISKRA_EINVAL before anything is launched
