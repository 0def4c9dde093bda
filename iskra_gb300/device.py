"""Device context: one grid, its species, fields, Poisson solver, MCC sets and
circuit on one GB300, driven through the C ABI of libiskra_gpu.so.

Arrays crossing this boundary use the reference's (Julia) layout: column-major
float64 node arrays (nx, ny), particle matrices (np, 2) / (np, 3).
"""
from __future__ import annotations

import ctypes
import os
from ctypes import byref, c_double, c_int, c_int64, c_uint64, c_void_p

import numpy as np

from . import _lib
from ._lib import check


def _f64(a, shape=None):
    a = np.asarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape, order="F")
    return np.asfortranarray(a)


def _ptr(a, t=_lib.dp):
    return None if a is None else a.ctypes.data_as(t)


def _mask(nodes, nx, ny):
    m = np.asarray(nodes, dtype=bool).reshape((nx, ny), order="F")
    return np.asfortranarray(m.astype(np.uint8))


class Context:
    """Owns an iskra_ctx (one CUDA stream)."""

    def __init__(self, nx, ny, dx, dy, bcs=(0, 0, 0, 0), stream: int = 0):
        self.lib = _lib.load()
        g = _lib.Grid(nx, ny, dx, dy, 0.0, 0.0, (ctypes.c_int32 * 4)(*[int(bool(b)) for b in bcs]))
        h = c_void_p()
        rc = self.lib.iskra_ctx_create(byref(g), stream, byref(h))
        if rc != 0:
            raise _lib.IskraError(rc, "iskra_ctx_create failed (is a CUDA device visible?)")
        self.h = h
        self.nx, self.ny, self.dx, self.dy = nx, ny, dx, dy
        self.bcs = tuple(bcs)
        self.species = []

    # -- plumbing --
    def _c(self, rc):
        return check(self.lib, self.h, rc)

    def close(self):
        if getattr(self, "h", None):
            self.lib.iskra_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        self._c(self.lib.iskra_sync(self.h))

    @property
    def stream(self) -> int:
        s = c_uint64()
        self._c(self.lib.iskra_stream(self.h, byref(s)))
        return s.value

    # -- species --
    def species_create(self, q, m, w0, capacity):
        sid = c_int()
        self._c(self.lib.iskra_species_create(self.h, q, m, w0, capacity, byref(sid)))
        self.species.append(sid.value)
        return sid.value

    def upload(self, sid, x, v, wg=None, ids=None):
        x = _f64(x)
        v = _f64(v)
        n = x.shape[0]
        wg = None if wg is None else _f64(wg)
        ids = None if ids is None else np.ascontiguousarray(ids, dtype=np.uint32)
        self._c(self.lib.iskra_species_upload(self.h, sid, _ptr(x), _ptr(v), _ptr(wg), _ptr(ids, _lib.u32p), n, n))

    def count(self, sid):
        n = c_int64()
        self._c(self.lib.iskra_species_count(self.h, sid, byref(n)))
        return n.value

    def download(self, sid, out=None):
        """Live particles (x, v, id).  out = (x (ld, 2), v (ld, 3), id (ld,)),
        Fortran-ordered float64 / uint32 (e.g. views of pinned host memory),
        receives them in place; views of its first np rows are returned."""
        if out is not None:
            x, v, ids = out
            cap = x.shape[0]
            if (x.shape != (cap, 2) or v.shape != (cap, 3) or ids.shape != (cap,) or not x.flags.f_contiguous
                    or not v.flags.f_contiguous or x.dtype != np.float64 or v.dtype != np.float64
                    or ids.dtype != np.uint32):
                raise ValueError("out must be (x (ld,2) F float64, v (ld,3) F float64, id (ld,) uint32)")
            got = c_int64()
            self._c(self.lib.iskra_species_download(self.h, sid, _ptr(x), _ptr(v), None, _ptr(ids, _lib.u32p), cap,
                                                    byref(got)))
            n = got.value
            return x[:n], v[:n], ids[:n]
        n = self.count(sid)
        cap = max(n, 1)
        x = np.zeros((cap, 2), order="F")
        v = np.zeros((cap, 3), order="F")
        ids = np.zeros(cap, dtype=np.uint32)
        got = c_int64()
        self._c(self.lib.iskra_species_download(self.h, sid, _ptr(x), _ptr(v), None, _ptr(ids, _lib.u32p), cap,
                                                byref(got)))
        n = got.value
        return np.asfortranarray(x[:n]), np.asfortranarray(v[:n]), ids[:n].copy()

    def set_boundary(self, sid, mode_x, mode_y):
        self._c(self.lib.iskra_species_set_boundary(self.h, sid, mode_x, mode_y))

    def absorbed(self, sid):
        a = (c_int64 * 4)()
        self._c(self.lib.iskra_species_absorbed(self.h, sid, a))
        return list(a)

    def sort(self, sid):
        self._c(self.lib.iskra_species_sort(self.h, sid))

    # -- surface tracker --
    def tracker_create(self, default_kind=_lib.SURF_ABSORB):
        self._c(self.lib.iskra_tracker_create(self.h, default_kind))

    def tracker_add_surface(self, nodes, kind, sigma_dof=0, area=0.0):
        """Edges with both end nodes in `nodes` (bool (nx, ny)) become surface
        `kind`; returns the surface index."""
        m = _mask(nodes, self.nx, self.ny)
        f = c_int(-1)
        self._c(self.lib.iskra_tracker_add_surface(self.h, _ptr(m, _lib.u8p), kind, sigma_dof, area, byref(f)))
        return f.value

    # -- particle sources --
    def source_create(self, sid, rate, wx, wv, dx=None, dv=None):
        """MaxwellianSource{2,3}(rate, wx, wv; dx, dv) feeding species sid."""
        arr = lambda a, n: np.ascontiguousarray(np.broadcast_to(np.asarray(a, float).ravel(), (n,)))
        wx_, wv_ = arr(wx, 2), arr(wv, 3)
        dx_ = arr(dx if dx is not None else 0.0, 2)
        dv_ = arr(dv if dv is not None else 0.0, 3)
        k = c_int(-1)
        self._c(self.lib.iskra_source_create(self.h, sid, float(rate), _ptr(wx_), _ptr(dx_), _ptr(wv_), _ptr(dv_),
                                             byref(k)))
        return k.value

    def source_sample(self, src, dt, seed=0):
        self._c(self.lib.iskra_source_sample(self.h, src, dt, seed))

    def source_every_step(self, src, on=True):
        self._c(self.lib.iskra_source_set_every_step(self.h, src, int(bool(on))))

    # -- DSMC --
    def dsmc_create(self, source, target, g, sigma):
        g_ = np.ascontiguousarray(g, float)
        s_ = np.ascontiguousarray(sigma, float)
        k = c_int(-1)
        self._c(self.lib.iskra_dsmc_create(self.h, source, target, _ptr(g_), _ptr(s_), len(g_), byref(k)))
        return k.value

    def dsmc_perform(self, k, dt, seed=0, step=0):
        self._c(self.lib.iskra_dsmc_perform(self.h, k, dt, seed, step))

    def dsmc_state(self, k):
        """(collisions_remaining, ν) per cell as (nx, ny) arrays."""
        rem = np.zeros((self.nx, self.ny), order="F")
        nu = np.zeros((self.nx, self.ny), dtype=np.uint32, order="F")
        self._c(self.lib.iskra_dsmc_state(self.h, k, _ptr(rem), _ptr(nu, _lib.u32p)))
        return rem, nu

    def tracker_hits(self, surface, sid):
        n = c_int64(0)
        self._c(self.lib.iskra_tracker_hits(self.h, surface, sid, byref(n)))
        return n.value

    # -- fields --
    def upload_E(self, E):
        E = _f64(E, (self.nx, self.ny, 3))
        self._c(self.lib.iskra_field_upload_E(self.h, _ptr(E)))

    def field(self, which, out=None):
        """ρ, ϕ or E as a Julia-layout FP64 array; `out` (Fortran-ordered, e.g.
        a view of pinned host memory) receives it in place when given."""
        shape = (self.nx, self.ny, 3) if which == _lib.FIELD_E else (self.nx, self.ny)
        if out is None:
            out = np.zeros(shape, order="F")
        elif out.shape != shape or out.dtype != np.float64 or not out.flags.f_contiguous:
            raise ValueError(f"out must be a Fortran-ordered float64 array of shape {shape}")
        self._c(self.lib.iskra_field_download(self.h, which, _ptr(out)))
        return out

    def field_async(self, which, out):
        """Non-blocking field download into `out` (Fortran-ordered float64, best
        a view of pinned host memory); valid after the next sync()."""
        shape = (self.nx, self.ny, 3) if which == _lib.FIELD_E else (self.nx, self.ny)
        if out.shape != shape or out.dtype != np.float64 or not out.flags.f_contiguous:
            raise ValueError(f"out must be a Fortran-ordered float64 array of shape {shape}")
        self._c(self.lib.iskra_field_download_async(self.h, which, _ptr(out)))
        return out

    def advance(self, sid, dt):
        self._c(self.lib.iskra_advance(self.h, sid, dt))

    def advance_all(self, dt):
        self._c(self.lib.iskra_advance_all(self.h, dt))

    def density(self, sid):
        out = np.zeros((self.nx, self.ny), order="F")
        self._c(self.lib.iskra_density(self.h, sid, _ptr(out)))
        return out

    def finalize(self, sid):
        """density(species) kept on the device (consumes the deposit accumulator)."""
        self._c(self.lib.iskra_density(self.h, sid, None))

    def charge_density(self):
        self._c(self.lib.iskra_charge_density(self.h))
        return self.field(_lib.FIELD_RHO)

    def set_background(self, rho_bg):
        if rho_bg is None:
            self._c(self.lib.iskra_set_background(self.h, None))
        else:
            a = _f64(rho_bg, (self.nx, self.ny))
            self._c(self.lib.iskra_set_background(self.h, _ptr(a)))

    # -- Poisson --
    def poisson_create(self, eps0):
        self._c(self.lib.iskra_poisson_create(self.h, eps0))

    def apply_dirichlet(self, nodes, phi0):
        m = _mask(nodes, self.nx, self.ny)
        self._c(self.lib.iskra_poisson_apply_dirichlet(self.h, _ptr(m, _lib.u8p), phi0))

    def apply_periodic(self, axis):
        self._c(self.lib.iskra_poisson_apply_periodic(self.h, axis))

    def add_dof(self):
        d = c_int()
        self._c(self.lib.iskra_poisson_add_dof(self.h, byref(d)))
        return d.value

    def apply_neumann(self, nodes, dof, gauss=False):
        """apply_neumann; gauss=True: the rows in stencil units with σ in C/m^2
        (iskra_poisson_apply_neumann_gauss)."""
        m = _mask(nodes, self.nx, self.ny)
        f = self.lib.iskra_poisson_apply_neumann_gauss if gauss else self.lib.iskra_poisson_apply_neumann
        self._c(f(self.h, _ptr(m, _lib.u8p), dof))

    def set_sigma(self, dof, value):
        self._c(self.lib.iskra_poisson_set_sigma(self.h, dof, value))

    def get_sigma(self, dof):
        v = c_double()
        self._c(self.lib.iskra_poisson_get_sigma(self.h, dof, byref(v)))
        return v.value

    def drive_dirichlet(self, nodes, amp, freq, phase=0.0, dc=0.0):
        m = _mask(nodes, self.nx, self.ny)
        self._c(self.lib.iskra_poisson_drive_dirichlet(self.h, _ptr(m, _lib.u8p), amp, freq, phase, dc))

    def set_warm_start(self, mode):
        self._c(self.lib.iskra_poisson_set_warm_start(self.h, mode))

    def set_method(self, method):
        a = c_int()
        self._c(self.lib.iskra_poisson_set_method(self.h, method, byref(a)))
        return a.value

    def solve(self, rtol=1e-8, maxit=10000):
        it, rr = c_int(), c_double()
        self._c(self.lib.iskra_poisson_solve(self.h, rtol, maxit, byref(it), byref(rr)))
        return it.value, rr.value

    def solve_host(self, f, rtol=1e-8, maxit=10000):
        f = _f64(f, (self.nx, self.ny))
        phi = np.zeros((self.nx, self.ny), order="F")
        it, rr = c_int(), c_double()
        self._c(self.lib.iskra_poisson_solve_host(self.h, _ptr(f), rtol, maxit, _ptr(phi), byref(it), byref(rr)))
        return phi, it.value, rr.value

    def solve_info(self):
        it, rr = c_int(), c_double()
        self._c(self.lib.iskra_solve_info(self.h, byref(it), byref(rr)))
        return it.value, rr.value

    def poisson_residual(self, f, phi):
        """||b - A ϕ|| / ||b|| of a host potential for the right-hand side f (FP64, host)."""
        fa = _f64(f, (self.nx, self.ny))
        pa = _f64(phi, (self.nx, self.ny))
        rr = c_double()
        self._c(self.lib.iskra_poisson_residual(self.h, _ptr(fa), _ptr(pa), byref(rr)))
        return rr.value

    # -- MCC --
    def mcc_create(self, src, processes, gas_mass, gas_T, gas_n, gas_q=0.0, product=-1):
        """processes: list of (type, energy, eps_nodes, sigma_nodes)."""
        N = len(processes)
        types = (c_int * N)(*[int(p[0]) for p in processes])
        energies = (c_double * N)(*[float(p[1]) for p in processes])
        off = np.zeros(N + 1, dtype=np.int32)
        for k, p in enumerate(processes):
            off[k + 1] = off[k] + len(p[2])
        eps = np.ascontiguousarray(np.concatenate([np.asarray(p[2], float) for p in processes]))
        sig = np.ascontiguousarray(np.concatenate([np.asarray(p[3], float) for p in processes]))
        gn = _f64(gas_n, (self.nx, self.ny))
        msg = c_double()
        mid = c_int()
        self._c(self.lib.iskra_mcc_create(self.h, src, N, types, energies, _ptr(off, _lib.i32p), _ptr(eps), _ptr(sig),
                                          gas_mass, gas_T, gas_q, _ptr(gn), product, byref(msg), byref(mid)))
        return mid.value, msg.value

    def mcc_perform(self, mid, dt, seed, step):
        self._c(self.lib.iskra_mcc_perform(self.h, mid, dt, seed, step))

    def mcc_counts(self, mid, nproc):
        a = (c_int64 * nproc)()
        self._c(self.lib.iskra_mcc_counts(self.h, mid, a))
        return list(a)

    def mcc_sigma(self, mid, process, energies):
        """σ of one process at the given energies (eV), as the MCC kernels evaluate it."""
        e = np.ascontiguousarray(energies, dtype=np.float64)
        out = np.zeros(len(e))
        self._c(self.lib.iskra_mcc_sigma(self.h, mid, process, _ptr(e), len(e), _ptr(out)))
        return out

    # -- circuit --
    def circuit_create(self, R, L, C, amp, freq, dc, sigma_dof, pos_nodes, neg_nodes, area, sigma_scale=1.0):
        pm = _mask(pos_nodes, self.nx, self.ny)
        nm = _mask(neg_nodes, self.nx, self.ny)
        self._c(self.lib.iskra_circuit_create(self.h, R, L, C, amp, freq, dc, sigma_dof, _ptr(pm, _lib.u8p),
                                              _ptr(nm, _lib.u8p), area, sigma_scale))

    def circuit_advance(self, dt):
        self._c(self.lib.iskra_circuit_advance(self.h, dt))

    def circuit_state(self):
        s = (c_double * 5)()
        self._c(self.lib.iskra_circuit_state(self.h, s))
        return dict(zip(("t", "i", "q", "sigma", "vext"), list(s)))

    # -- whole step --
    def step(self, dt, nsteps=1, seed=0, rtol=1e-8):
        self._c(self.lib.iskra_step(self.h, dt, nsteps, seed, rtol))

    def kernel_launches(self):
        n = c_uint64()
        self._c(self.lib.iskra_kernel_launches(self.h, byref(n)))
        return n.value

    def write_openpmd(self, prefix, iteration, time, dt, species_names=None, particles=True):
        """new_iteration + save_record of every record: <prefix>/hdf5/data<iteration>.h5."""
        names = None
        if species_names is not None:
            names = (ctypes.c_char_p * len(species_names))(*[s.encode() for s in species_names])
        self._c(self.lib.iskra_write_openpmd(self.h, str(prefix).encode(), int(iteration), float(time), float(dt),
                                             names, int(bool(particles))))
        return os.path.join(str(prefix), "hdf5", f"data{int(iteration)}.h5")

    def set_sort_every(self, every):
        self._c(self.lib.iskra_set_sort_every(self.h, every))

    def set_tile(self, cells):
        self._c(self.lib.iskra_set_tile(self.h, int(cells)))

    def tile(self):
        t = c_int()
        self._c(self.lib.iskra_get_tile(self.h, byref(t)))
        return t.value

    def autotune(self, dt, trial=64, seed=0, rtol=1e-8):
        """Push tile size and sort cadence tuned together on this run:
        (tile, sort-period factor, ms per step, {(tile, factor): ms}, cached)."""
        t, f, ms, cached = c_int(), c_double(), c_double(), c_int()
        allv = (c_double * 12)()
        self._c(self.lib.iskra_autotune(self.h, dt, trial, seed, rtol, byref(t), byref(f), byref(ms), allv,
                                        byref(cached)))
        grid = {(tile, fac): allv[4 * k + j] for k, tile in enumerate((8, 16, 32))
                for j, fac in enumerate((0.5, 1.0, 2.0, 4.0))}
        return t.value, f.value, ms.value, (None if cached.value else grid), bool(cached.value)

    def autotune_sort(self, dt, trial=64, seed=0, rtol=1e-8):
        """Returns (chosen factor on the speed-based sort periods, ms per step)."""
        f, ms = c_double(), c_double()
        self._c(self.lib.iskra_autotune_sort(self.h, dt, trial, seed, rtol, byref(f), byref(ms)))
        return f.value, ms.value

    # -- learned warm start of CG solves --
    def lws_create(self, capacity=0, seed=0):
        self._c(self.lib.iskra_lws_create(self.h, capacity, seed))

    def lws_destroy(self):
        self._c(self.lib.iskra_lws_destroy(self.h))

    def lws_set_mode(self, harvest=False, use=False, smooth=4):
        self._c(self.lib.iskra_lws_set_mode(self.h, int(harvest), int(use), int(smooth)))

    def lws_info(self):
        pairs, npar, solves, warm, alpha, ratio = c_int(), c_int(), c_int64(), c_int64(), c_double(), c_double()
        self._c(self.lib.iskra_lws_info(self.h, byref(pairs), byref(npar), byref(solves), byref(warm),
                                        byref(alpha), byref(ratio)))
        return dict(pairs=pairs.value, nparams=npar.value, solves=solves.value, warm_solves=warm.value,
                    mean_alpha=alpha.value, mean_ratio=ratio.value)

    def lws_eval(self):
        loss, zero = c_double(), c_double()
        self._c(self.lib.iskra_lws_eval(self.h, byref(loss), byref(zero)))
        return loss.value, zero.value

    def lws_weights(self, new=None):
        n = self.lws_info()["nparams"]
        out = np.empty(n, np.float32)
        w_in = None
        if new is not None:
            w_in = np.ascontiguousarray(new, np.float32)
            assert w_in.size == n
        self._c(self.lib.iskra_lws_weights(self.h, _ptr(out, _lib.f32p),
                                           _ptr(w_in, _lib.f32p) if w_in is not None else None))
        return out

    def lws_forward(self, img):
        """img: (ny, nx) float32 (x fastest); returns the (ny, nx) output."""
        x = np.ascontiguousarray(img, np.float32).reshape(self.ny, self.nx)
        y = np.empty_like(x)
        self._c(self.lib.iskra_lws_forward(self.h, _ptr(x, _lib.f32p), _ptr(y, _lib.f32p)))
        return y

    def lws_loss_grad(self, img, target):
        x = np.ascontiguousarray(img, np.float32).reshape(self.ny, self.nx)
        t = np.ascontiguousarray(target, np.float32).reshape(self.ny, self.nx)
        g = np.empty(self.lws_info()["nparams"], np.float32)
        loss = c_double()
        self._c(self.lib.iskra_lws_loss_grad(self.h, _ptr(x, _lib.f32p), _ptr(t, _lib.f32p), byref(loss),
                                             _ptr(g, _lib.f32p)))
        return loss.value, g

    def lws_train(self, iters, lr=1e-3, seed=0):
        loss = c_double()
        self._c(self.lib.iskra_lws_train(self.h, iters, lr, seed, byref(loss)))
        return loss.value


class Ensemble:
    """Batched independent runs of a configured template Context (the
    GPUEnsemble of the batched configuration): per-run particles, fields,
    MCC seeds and drive amplitudes; one step advances every run.  The
    template must stay open while the ensemble lives."""

    def __init__(self, template: Context, nruns: int, capacity_per_run: int):
        self.lib = template.lib
        self.template = template
        h = c_void_p()
        rc = self.lib.iskra_ens_create(template.h, nruns, capacity_per_run, byref(h))
        if rc != 0:
            raise _lib.IskraError(rc, self.lib.iskra_last_error(template.h).decode())
        self.h = h
        self.R = nruns
        self.nx, self.ny = template.nx, template.ny

    def _c(self, rc):
        if rc != _lib.ISKRA_OK:
            msg = self.lib.iskra_ens_last_error(self.h)
            raise _lib.IskraError(rc, msg.decode() if msg else "")
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.lib.iskra_ens_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_seeds(self, seeds):
        a = (c_uint64 * self.R)(*[int(s) for s in seeds])
        self._c(self.lib.iskra_ens_set_seeds(self.h, a))

    def set_drive_amplitude(self, group, amps):
        a = np.ascontiguousarray(amps, dtype=np.float64)
        self._c(self.lib.iskra_ens_set_drive_amplitude(self.h, group, _ptr(a)))

    def upload(self, run, sid, x, v, ids=None):
        x = _f64(x)
        v = _f64(v)
        n = x.shape[0]
        ids = None if ids is None else np.ascontiguousarray(ids, dtype=np.uint32)
        self._c(self.lib.iskra_ens_upload(self.h, run, sid, _ptr(x), _ptr(v), _ptr(ids, _lib.u32p), n, n))

    def count(self, run, sid):
        n = c_int64()
        self._c(self.lib.iskra_ens_count(self.h, run, sid, byref(n)))
        return n.value

    def download(self, run, sid):
        n = self.count(run, sid)
        cap = max(n, 1)
        x = np.zeros((cap, 2), order="F")
        v = np.zeros((cap, 3), order="F")
        ids = np.zeros(cap, dtype=np.uint32)
        got = c_int64()
        self._c(self.lib.iskra_ens_download(self.h, run, sid, _ptr(x), _ptr(v), _ptr(ids, _lib.u32p), cap,
                                            byref(got)))
        n = got.value
        return np.asfortranarray(x[:n]), np.asfortranarray(v[:n]), ids[:n].copy()

    def step(self, dt, nsteps=1):
        self._c(self.lib.iskra_ens_step(self.h, dt, nsteps))

    def sync(self):
        self._c(self.lib.iskra_ens_sync(self.h))

    def mcc_counts(self, run, mid, nproc):
        a = (c_uint64 * nproc)()
        self._c(self.lib.iskra_ens_mcc_counts(self.h, run, mid, a))
        return list(a)

    def field(self, run, which):
        shape = (self.nx, self.ny, 3) if which == _lib.FIELD_E else (self.nx, self.ny)
        out = np.zeros(shape, order="F")
        self._c(self.lib.iskra_ens_field(self.h, run, which, _ptr(out)))
        return out

    def set_compact_every(self, every):
        self._c(self.lib.iskra_ens_set_compact_every(self.h, every))
