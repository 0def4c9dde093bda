"""openPMD/HDF5 records (Diagnostics/src/hdf5.jl:47-101) written by
iskra_write_openpmd and read back by the independent reader tests/h5read.py
(every checksum verified): the field datasets equal the context's own
downloads, the particle records its particles, the openPMD metadata the
reference's (openpmd/root.jl, fields.jl, particles.jl).  No HDF5 library
exists on these machines, so the files are not verified by libhdf5."""
import numpy as np
import pytest

import h5read
from test_gpu_discharge import EPS0, KB, M_AR, ME, QE, argon_tables

pytestmark = pytest.mark.gpu


def test_openpmd_records_round_trip(lib, tmp_path):
    from iskra_gb300.device import Context
    nx, ny, gap = 65, 2, 0.025
    dx = gap / (nx - 1)
    rng = np.random.default_rng(4)
    n0 = 5000
    w = 1e15 * gap * dx / n0
    ctx = Context(nx, ny, dx, dx)
    se = ctx.species_create(-QE, ME, w, 4 * n0)
    si = ctx.species_create(QE, M_AR, w, 4 * n0)
    for s, T, m in ((se, 4.0, ME), (si, 0.03, M_AR)):
        ctx.set_boundary(s, lib.BND_DISCARD, lib.BND_WRAP)
        x = np.column_stack([rng.uniform(0, gap, n0), rng.uniform(0, dx, n0)])
        ctx.upload(s, x, rng.standard_normal((n0, 3)) * np.sqrt(2 * T * QE / m))
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    left = np.zeros((nx, ny), bool)
    left[0, :] = True
    right = np.zeros((nx, ny), bool)
    right[-1, :] = True
    dof = ctx.add_dof()
    ctx.apply_neumann(left, dof, gauss=True)
    ctx.apply_dirichlet(right, 0.0)
    ctx.circuit_create(50.0, 1e-6, 1e-9, 300.0, 13.56e6, 0.0, dof, left, right, dx, 1.0)
    eps, el, ex, iz, cx = argon_tables()
    gas_n = np.full((nx, ny), 3.0 / (KB * 300.0))
    me_, _ = ctx.mcc_create(se, [(lib.MCC_ELASTIC_ISOTROPIC, 0.0, eps, el), (lib.MCC_EXCITATION, 11.5, eps, ex),
                                 (lib.MCC_IONIZATION, 15.76, eps, iz)], M_AR, 300.0, gas_n, product=si)
    ctx.step(7.4e-11, 20, seed=3, rtol=1e-10)
    ctx.sync()
    path = ctx.write_openpmd(str(tmp_path), 20, 20 * 7.4e-11, 7.4e-11, ["e", "Ar+"])
    rho, phi, E = ctx.field(lib.FIELD_RHO), ctx.field(lib.FIELD_PHI), ctx.field(lib.FIELD_E)
    ne, ni = ctx.density(se), ctx.density(si)
    parts = {"e": ctx.download(se), "Ar+": ctx.download(si)}
    st = ctx.circuit_state()
    counts = ctx.mcc_counts(me_, 3)
    ctx.close()

    f = h5read.File(path)
    root = f.get("/")
    assert root.attrs["openPMD"] == "1.1.0" and root.attrs["openPMDextension"] == 1
    assert root.attrs["basePath"] == "/data/%T" and root.attrs["meshesPath"] == "fields/"
    assert root.attrs["iterationEncoding"] == "fileBased" and root.attrs["iterationFormat"] == "data%T.h5"
    it = f.get("/data/20")
    assert it.attrs["dt"] == 7.4e-11 and abs(it.attrs["time"] - 20 * 7.4e-11) < 1e-24
    base = "/data/20/fields/"
    # fields in Julia memory order: HDF5 dims (ny, nx), x fastest
    def as_julia(a):
        return np.asarray(a).reshape(-1).reshape((nx, ny), order="F")
    assert np.array_equal(as_julia(f.read(base + "rho")), rho)
    assert np.array_equal(as_julia(f.read(base + "phi")), phi)
    for k, c in enumerate("xyz"):
        assert np.array_equal(as_julia(f.read(base + "E/" + c)), E[:, :, k])
    assert np.array_equal(as_julia(f.read(base + "ne")), ne)
    assert np.array_equal(as_julia(f.read(base + "nAr+")), ni)
    assert f.read(base + "rho").shape == (ny, nx)
    rec = f.get(base + "phi")
    assert list(rec.attrs["unitDimension"]) == [2, 1, -3, -1, 0, 0, 0]
    assert list(rec.attrs["gridSpacing"]) == [dx, dx] and rec.attrs["dataOrder"] == "C"
    assert rec.attrs["geometry"] == "cartesian" and rec.attrs["unitSI"] == 1.0
    # accepted collisions per node: their total is the accepted count of the steps
    nu_tot = sum(f.read(base + f"nuMCC-e-{k + 1}").sum() for k in range(3))
    assert nu_tot == sum(counts) > 0
    # circuit probes
    assert f.read(base + "I1")[0] == st["i"] and f.read(base + "Q1")[0] == st["q"]
    assert f.read(base + "Vext")[0] == st["vext"]
    # particles
    for name, (x, v, ids) in parts.items():
        pb = f"/data/20/particles/{name}/"
        o = np.argsort(ids)
        fo = np.argsort(f.read(pb + "id"))
        assert np.array_equal(f.read(pb + "id")[fo], ids[o].astype(float))
        assert np.array_equal(f.read(pb + "position/x")[fo], x[o, 0])
        assert np.array_equal(f.read(pb + "position/y")[fo], x[o, 1])
        m = ME if name == "e" else M_AR
        for k, c in enumerate("xyz"):
            assert np.allclose(f.read(pb + "momentum/" + c)[fo], m * v[o, k], rtol=1e-15, atol=0)
        assert f.get(pb + "charge").attrs["value"] == (-QE if name == "e" else QE)
        assert f.get(pb + "mass").attrs["value"] == m
        assert f.get(pb + "weighting").attrs["macroWeighted"] == 1
    # a corrupted byte in an object header fails its checksum
    raw = bytearray(open(path, "rb").read())
    at = raw.find(b"OHDR", 100)
    raw[at + 8] ^= 0xFF
    bad = tmp_path / "bad.h5"
    bad.write_bytes(bytes(raw))
    with pytest.raises(h5read.H5Error):
        g = h5read.File(str(bad))
        for p in ("/data/20/fields/rho", "/data/20/fields/phi", "/data/20/particles/e/id"):
            g.get(p)
        g.get("/data/20/fields/E/x")
        g.get("/data/20/fields/ne")
        g.get("/data/20/fields/nAr+")
        raise AssertionError("corruption not detected")
