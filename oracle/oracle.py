"""FP64 CPU oracle for iskra's electrostatic PIC step -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker.  The product path
(``iskra_gb300`` -> ``libiskra_gpu.so``) never imports it.

Two parts:
  * ctypes bindings of ``liboracle.so`` (``iskra_oracle.c``): particle_cell,
    CIC gather/deposit, Boris push, wrap!/discard!, cell volume, E field,
    MCC, circuit -- each a restatement of one Julia function, cited there.
  * ``PoissonOracle``: the FP64 Poisson operator assembled exactly as
    ``FiniteDifferenceMethod/src/generalized_poisson.jl`` does
    (``create_generalized_poisson_solver`` :34-68, ``apply_dirichlet`` :205-215,
    ``add_new_dof`` :217-230, ``apply_neumann`` :235-269, ``apply_periodic``
    :286-324), solved by sparse LU (the reference uses dense ``A\\b``, :201-203,
    which is infeasible beyond ~100^2 nodes; LU is the same direct method).
    When no row pins the potential the matrix is singular; the oracle then
    solves the bordered system [A 1; 1' 0] (mean-zero gauge).  E = -grad(phi)
    is independent of that gauge.

Pin status: Poisson/E-field pinned by the reference's own parallel-plate test
(FiniteDifferenceMethod/test/runtests.jl:8-22, restated in
tests/test_oracle_cpu.py); everything else parity unpinned (analytic
known answers only; Julia is not available to run the reference).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_int, c_int64, c_uint32, c_uint64

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

dp = POINTER(c_double)
ip = POINTER(c_int)
i64p = POINTER(c_int64)
u32p = POINTER(c_uint32)


def build():
    """Compile liboracle.so in place (gcc + make)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.orc_particle_cell.argtypes = [c_double, c_double, c_double, c_double, i64p, i64p, dp, dp]
        L.orc_cell_volume.argtypes = [c_int, c_int, c_double, c_double, ip, dp]
        L.orc_grid_to_particle.argtypes = [c_int, c_int, c_double, c_double, dp, c_int64, c_int64, dp, dp, c_int64]
        L.orc_grid_to_particle.restype = c_int64
        L.orc_push_cartesian.argtypes = [c_int64, c_int64, dp, dp, dp, dp, c_int64, c_double, c_double]
        L.orc_discard.argtypes = [c_int64, c_int64, dp, dp, dp, u32p, c_double, c_int, c_int, c_double, c_double, i64p, i64p]
        L.orc_discard.restype = c_int64
        L.orc_wrap.argtypes = [c_int64, c_int64, dp, c_int, c_int, c_double, c_double]
        L.orc_particle_to_grid.argtypes = [c_int, c_int, c_double, c_double, c_int64, c_int64, dp, dp, c_double, dp]
        L.orc_particle_to_grid.restype = c_int64
        L.orc_particle_to_grid_omp.argtypes = [c_int, c_int, c_double, c_double, c_int64, c_int64, dp, c_double, dp, c_int]
        L.orc_particle_to_grid_omp.restype = c_int64
        L.orc_electric_field.argtypes = [c_int, c_int, c_double, c_double, dp, dp]
        L.orc_advance_circuit.argtypes = [c_double, c_double, c_double, dp, c_double, c_double, c_double]
        L.orc_sigma.argtypes = [dp, dp, c_int, c_double]
        L.orc_sigma.restype = c_double
        L.orc_mass_ev.argtypes = [c_double]
        L.orc_mass_ev.restype = c_double
        L.orc_thermal_speed.argtypes = [c_double, c_double]
        L.orc_thermal_speed.restype = c_double
        L.orc_mcc_max_sigma_g.argtypes = [c_int, ip, dp, dp, c_double]
        L.orc_mcc_max_sigma_g.restype = c_double
        L.orc_isotropic_scattering.argtypes = [dp, c_double, c_double, dp]
        L.orc_diffuse_reflection.argtypes = [dp, c_double, c_double, dp]
        L.orc_mcc_perform.argtypes = [
            c_int, c_int, c_double, c_double, dp, dp, c_int, ip, dp, ip, dp, dp, c_double, dp,
            c_double, dp, dp, i64p, c_int64, c_double, c_double, c_double, dp, dp, i64p, c_int64,
            c_double, c_double, c_double, c_double, c_uint64, i64p, dp]
        L.orc_mcc_perform.restype = c_int
        L.orc_fill_uniform.argtypes = [c_uint64, c_int64, dp]
        L.orc_fill_normal.argtypes = [c_uint64, c_int64, dp]
        L.orc_num_threads.restype = c_int
        _LIB = L
    return _LIB


def _p(a, t=dp):
    return a.ctypes.data_as(t) if a is not None else None


def _f64(a):
    return np.require(a, dtype=np.float64, requirements=["F", "A", "W"])


# ----------------------------------------------------------------------------
# particle / grid operations (iskra_oracle.c restatements)
# ----------------------------------------------------------------------------

def particle_cell(x, y, dx, dy):
    i, j = c_int64(), c_int64()
    hx, hy = c_double(), c_double()
    lib().orc_particle_cell(x, y, dx, dy, ctypes.byref(i), ctypes.byref(j), ctypes.byref(hx), ctypes.byref(hy))
    return i.value, j.value, hx.value, hy.value


def cell_volume(nx, ny, dx, dy, bcs=(0, 0, 0, 0)):
    V = np.zeros((nx, ny), order="F")
    b = np.asarray(bcs, dtype=np.int32)
    lib().orc_cell_volume(nx, ny, dx, dy, _p(b, ip), _p(V))
    return V


def grid_to_particle(E, dx, dy, x):
    """E: (nx,ny,3) F-order; x: (np,2) F-order.  Returns pu (np,3)."""
    E = _f64(E)
    x = _f64(x)
    nx, ny, _ = E.shape
    n = x.shape[0]
    pu = np.zeros((n, 3), order="F")
    bad = lib().orc_grid_to_particle(nx, ny, dx, dy, _p(E), n, n, _p(x), _p(pu), n)
    if bad:
        raise IndexError(f"particle {bad} outside the grid")
    return pu


def push_cartesian(x, v, Ep, Bp, qm, dt):
    """In-place Boris push of (np,2) x and (np,3) v."""
    n = x.shape[0]
    assert x.flags.f_contiguous and v.flags.f_contiguous
    Ep = _f64(Ep)
    Bp = None if Bp is None else _f64(Bp)
    lib().orc_push_cartesian(n, n, _p(x), _p(v), _p(Ep), _p(Bp), n, qm, dt)


def discard(x, v, wg, pid, w0, dim, n_nodes, dh, origin=0.0):
    """discard! on the first np rows; returns (np_new, removed_lo, removed_hi)."""
    n = x.shape[0]
    lo, hi = c_int64(0), c_int64(0)
    npn = lib().orc_discard(n, n, _p(x), _p(v), _p(wg), _p(pid, u32p), w0, dim, n_nodes, dh, origin,
                            ctypes.byref(lo), ctypes.byref(hi))
    return npn, lo.value, hi.value


def wrap(x, dim, n_nodes, dh, origin=0.0):
    n = x.shape[0]
    lib().orc_wrap(n, n, _p(x), dim, n_nodes, dh, origin)


def particle_to_grid(nx, ny, dx, dy, x, wg=None, w0=1.0):
    x = _f64(x)
    n = x.shape[0]
    u = np.zeros((nx, ny), order="F")
    wgp = None if wg is None else _f64(wg)
    bad = lib().orc_particle_to_grid(nx, ny, dx, dy, n, n, _p(x), _p(wgp), w0, _p(u))
    if bad:
        raise IndexError(f"particle {bad} outside the grid")
    return u


def particle_to_grid_omp(nx, ny, dx, dy, x, w0, nthreads):
    n = x.shape[0]
    u = np.zeros((nx, ny), order="F")
    bad = lib().orc_particle_to_grid_omp(nx, ny, dx, dy, n, n, _p(x), w0, _p(u), nthreads)
    if bad:
        raise IndexError(f"particle {bad} outside the grid")
    return u


def density(nx, ny, dx, dy, x, w0, bcs):
    """density(species, grid) = particle_to_grid(wg) ./ cell_volume (kinetic.jl:53)."""
    return particle_to_grid(nx, ny, dx, dy, x, None, w0) / cell_volume(nx, ny, dx, dy, bcs)


def electric_field(phi, dx, dy):
    phi = _f64(phi)
    nx, ny = phi.shape
    E = np.zeros((nx, ny, 3), order="F")
    lib().orc_electric_field(nx, ny, dx, dy, _p(phi), _p(E))
    return E


def advance_circuit(R, L, C, state, vext, vsrc, dt):
    s = np.asarray(state, dtype=np.float64).copy()
    lib().orc_advance_circuit(R, L, C, _p(s), vext, vsrc, dt)
    return s


def sigma(eps, sig, e):
    eps = np.ascontiguousarray(eps, dtype=np.float64)
    sig = np.ascontiguousarray(sig, dtype=np.float64)
    return lib().orc_sigma(_p(eps), _p(sig), len(eps), e)


def mass_ev(m):
    return lib().orc_mass_ev(m)


def thermal_speed(T, m):
    return lib().orc_thermal_speed(T, m)


def mcc_max_sigma_g(tables, m_source):
    off = np.zeros(len(tables) + 1, dtype=np.int32)
    for k, (e, s) in enumerate(tables):
        off[k + 1] = off[k] + len(e)
    eps = np.ascontiguousarray(np.concatenate([np.asarray(e, float) for e, _ in tables]))
    sig = np.ascontiguousarray(np.concatenate([np.asarray(s, float) for _, s in tables]))
    return lib().orc_mcc_max_sigma_g(len(tables), _p(off, ip), _p(eps), _p(sig), m_source)


def isotropic_scattering(v, u1, u2):
    v = np.ascontiguousarray(v, dtype=np.float64)
    out = np.zeros(3)
    lib().orc_isotropic_scattering(_p(v), u1, u2, _p(out))
    return out


def diffuse_reflection(v, u1, u2):
    v = np.ascontiguousarray(v, dtype=np.float64)
    out = np.zeros(3)
    lib().orc_diffuse_reflection(_p(v), u1, u2, _p(out))
    return out


def uniform(seed, n):
    out = np.zeros(n)
    lib().orc_fill_uniform(seed, n, _p(out))
    return out


def normal(seed, n):
    out = np.zeros(n)
    lib().orc_fill_normal(seed, n, _p(out))
    return out


MCC_TYPES = {"elastic_isotropic": 0, "elastic_backward": 1, "inelastic_backward": 2,
             "excitation": 3, "ionization": 4}


class MCCOracle:
    """MonteCarloCollisions + PIC.perform! (Chemistry/src/mcc.jl:18-51,231-289)."""

    def __init__(self, processes, m_source, q_source, w0_source, gas_mass, gas_T, gas_q=0.0,
                 product_w0=None):
        # processes: list of (type_name, energy, eps_nodes, sigma_nodes)
        self.N = len(processes)
        self.types = np.array([MCC_TYPES[p[0]] for p in processes], dtype=np.int32)
        self.energies = np.array([p[1] for p in processes], dtype=np.float64)
        self.off = np.zeros(self.N + 1, dtype=np.int32)
        for k, p in enumerate(processes):
            self.off[k + 1] = self.off[k] + len(p[2])
        self.eps = np.ascontiguousarray(np.concatenate([np.asarray(p[2], float) for p in processes]))
        self.sig = np.ascontiguousarray(np.concatenate([np.asarray(p[3], float) for p in processes]))
        self.m, self.q, self.w0 = m_source, q_source, w0_source
        self.gas_mass, self.gas_T, self.gas_q = gas_mass, gas_T, gas_q
        self.product_w0 = product_w0
        self.max_sigma_g = lib().orc_mcc_max_sigma_g(self.N, _p(self.off, ip), _p(self.eps), _p(self.sig), m_source)
        self.remainder = 0.0

    def perform(self, E, n_gas, dx, dy, dt, sx, sv, snp, seed, px=None, pv=None, pnp=0, nu=None):
        """Runs one MCC step in place on (cap,2)/(cap,3) F-order stores.
        Returns (np_source, np_product, counts[N])."""
        E = _f64(E)
        n_gas = _f64(n_gas)
        nx, ny = n_gas.shape
        snp_c = c_int64(snp)
        pnp_c = c_int64(pnp)
        rem = c_double(self.remainder)
        counts = np.zeros(self.N, dtype=np.int64)
        pw0 = self.product_w0 if self.product_w0 is not None else 1.0
        rc = lib().orc_mcc_perform(
            nx, ny, dx, dy, _p(E), _p(n_gas), self.N, _p(self.types, ip), _p(self.energies),
            _p(self.off, ip), _p(self.eps), _p(self.sig), self.max_sigma_g, ctypes.byref(rem), dt,
            _p(sx), _p(sv), ctypes.byref(snp_c), sx.shape[0], self.m, self.q, self.w0,
            _p(px), _p(pv), ctypes.byref(pnp_c), 0 if px is None else px.shape[0], pw0,
            self.gas_mass, self.gas_q, self.gas_T, seed, _p(counts, i64p), _p(nu))
        if rc == -2:
            raise AssertionError("collision probability exceeds bound (mcc.jl:244-246,272-279)")
        if rc == -1:
            raise MemoryError("species capacity exceeded")
        self.remainder = rem.value
        return snp_c.value, pnp_c.value, counts


# ----------------------------------------------------------------------------
# Poisson operator (generalized_poisson.jl) in 7-slot row form
# ----------------------------------------------------------------------------
# slot 0: self, 1: (i-1,j), 2: (i+1,j), 3: (i,j-1), 4: (i,j+1),
# 5: x-periodic partner ((1<->nx), j), 6: y-periodic partner (i, (1<->ny)).
# sigma columns are kept in a separate dense (nnodes x nsigma) block.

class PoissonOracle:
    def __init__(self, nx, ny, dx, dy, eps0, eps_r=None):
        """create_poisson_solver(grid::CartesianGrid{2}, ε0) -> generalized solver
        with εr = ones(nx+1, ny+1) (generalized_poisson.jl:27-30,34-68)."""
        self.nx, self.ny, self.dx, self.dy, self.eps0 = nx, ny, dx, dy, eps0
        self.er = np.ones((nx + 1, ny + 1)) if eps_r is None else np.asarray(eps_r, float)
        nn = nx * ny
        self.nn = nn
        C = np.zeros((nn, 7))
        I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        I = I.ravel(order="F")
        J = J.ravel(order="F")
        r = I + nx * J
        # i < nx: -1 self, +1 (i+1); i > 1: -1 self, +1 (i-1); same for j (:42-61)
        m = I < nx - 1
        C[r[m], 0] -= 1.0
        C[r[m], 2] += 1.0
        m = I > 0
        C[r[m], 0] -= 1.0
        C[r[m], 1] += 1.0
        m = J < ny - 1
        C[r[m], 0] -= 1.0
        C[r[m], 4] += 1.0
        m = J > 0
        C[r[m], 0] -= 1.0
        C[r[m], 3] += 1.0
        C /= dx ** 2  # A ./= grid.Δh[1]^2 (:65)
        self.C = C
        self.b = np.zeros(nn)
        self.rho_dof = np.ones(nn, dtype=bool)  # dofs[:ρ] = 1:nn (:41)
        self.sig_cols = np.zeros((nn, 0))       # A[ϕ, σ] block
        self.sig_b = []                         # b[σ]

    def _rc(self):
        nx, ny = self.nx, self.ny
        I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        return I.ravel(order="F"), J.ravel(order="F")

    def apply_periodic(self, axis):
        """apply_periodic(ps::PoissonSolver{:xy,2}, axis) (:286-324).  axis 1
        couples j=1 <-> j=ny (coefficient over Δx^2), axis 2 couples
        i=1 <-> i=nx (over Δy^2) -- the reference's axis naming."""
        nx, ny, er = self.nx, self.ny, self.er
        C = self.C
        if axis == 1:
            for j in (0, ny - 1):  # Julia iterates the tuple (1, ny)
                for i in range(nx):
                    r = i + nx * j
                    if j == ny - 1:
                        c = (0.5 * er[i + 1, j + 1] + 0.5 * er[i, j + 1]) / self.dx ** 2
                        C[r, 0] -= c
                        C[r, 6] += c
                    if j == 0:
                        c = (0.5 * er[i + 1, j] + 0.5 * er[i, j]) / self.dx ** 2
                        C[r, 0] -= c
                        C[r, 6] += c
        if axis == 2:
            for j in range(ny):
                for i in (0, nx - 1):  # Julia iterates the tuple (1, nx)
                    r = i + nx * j
                    if i == nx - 1:
                        c = (0.5 * er[i + 1, j + 1] + 0.5 * er[i + 1, j]) / self.dy ** 2
                        C[r, 0] -= c
                        C[r, 5] += c
                    if i == 0:
                        c = (0.5 * er[i, j] + 0.5 * er[i, j + 1]) / self.dy ** 2
                        C[r, 0] -= c
                        C[r, 5] += c

    def apply_dirichlet(self, nodes, phi0):
        """apply_dirichlet (:205-215): identity row, b = ϕ0, drop from ρ dofs."""
        sel = np.asarray(nodes, dtype=bool).ravel(order="F")
        self.C[sel, :] = 0.0
        self.C[sel, 0] = 1.0
        if self.sig_cols.shape[1]:
            self.sig_cols[sel, :] = 0.0
        self.b[sel] = phi0
        self.rho_dof[sel] = False

    def add_new_dof(self):
        """add_new_dof(ps, :σ) (:217-230): identity row, b = 0.  Returns 1-based dof."""
        self.sig_cols = np.concatenate([self.sig_cols, np.zeros((self.nn, 1))], axis=1)
        self.sig_b.append(0.0)
        return len(self.sig_b)

    def apply_neumann(self, nodes, dof, gauss=False):
        """apply_neumann(ps::PoissonSolver{:xy,2}, nodes, dof) (:235-269).
        gauss=True: the same rows in stencil units with σ in C/m^2 -- the edge
        row divided by Δx with σ coefficient 2/(ε0 Δx), the corner rows' σ
        coefficient divided by ε0 (the half/quarter-cell Gauss law; the
        declared consistent form of the library's
        iskra_poisson_apply_neumann_gauss)."""
        nodes = np.asarray(nodes, dtype=bool)
        nx, ny, er = self.nx, self.ny, self.er
        dx, dy = self.dx, self.dy
        ge = dx ** 2 if gauss else dx   # edge-row ϕ divisor
        gs = 1.0 / (self.eps0 * dx) if gauss else 1.0
        gc = 1.0 / self.eps0 if gauss else 1.0
        for (i, j) in zip(*np.nonzero(nodes)):
            a = nodes[i - 1, j] if i > 0 else False
            b = nodes[i + 1, j] if i < nx - 1 else False
            c = nodes[i, j - 1] if j > 0 else True
            d = nodes[i, j + 1] if j < ny - 1 else True
            r = i + nx * j
            if c == d == True and a == b == False:  # noqa: E712
                ip_ = i + 1 if i == 0 else i - 1
                self.C[r, :] = 0.0
                self.sig_cols[r, :] = 0.0
                self.C[r, 0] -= 2 * er[i, j] / ge
                self.C[r, 2 if ip_ == i + 1 else 1] += 2 * er[ip_, j] / ge
                self.sig_cols[r, dof - 1] += 2 * gs
            if c != d:
                ip_ = i + 1 if i == 0 else i - 1
                jp_ = j + 1 if c else j - 1
                self.C[r, :] = 0.0
                self.sig_cols[r, :] = 0.0
                self.C[r, 0] -= 4 * er[i, j] / (3 * dx ** 2)
                self.C[r, 0] -= 4 * er[i, j] / (3 * dy ** 2)
                self.C[r, 2 if ip_ == i + 1 else 1] += 4 * er[i, j] / (3 * dx ** 2)
                self.C[r, 4 if jp_ == j + 1 else 3] += 4 * er[i, j] / (3 * dy ** 2)
                self.sig_cols[r, dof - 1] += (2 / 3) * (dx + dy) / (dx * dy) * gc

    def set_sigma(self, dof, value):
        self.sig_b[dof - 1] = value

    def matrix(self):
        """Assembled sparse A over [nodes..., sigma dofs...]."""
        import scipy.sparse as sp
        nx, ny, nn = self.nx, self.ny, self.nn
        I, J = self._rc()
        r = I + nx * J
        cols = [r,
                np.where(I > 0, r - 1, r), np.where(I < nx - 1, r + 1, r),
                np.where(J > 0, r - nx, r), np.where(J < ny - 1, r + nx, r),
                np.where(I == 0, (nx - 1) + nx * J, I * 0 + nx * J),
                np.where(J == 0, I + nx * (ny - 1), I)]
        rows_l, cols_l, vals_l = [], [], []
        for s in range(7):
            m = self.C[:, s] != 0.0
            rows_l.append(r[m])
            cols_l.append(cols[s][m])
            vals_l.append(self.C[m, s])
        ns = self.sig_cols.shape[1]
        for k in range(ns):
            m = self.sig_cols[:, k] != 0.0
            rows_l.append(r[m])
            cols_l.append(np.full(m.sum(), nn + k))
            vals_l.append(self.sig_cols[m, k])
            rows_l.append(np.array([nn + k]))
            cols_l.append(np.array([nn + k]))
            vals_l.append(np.array([1.0]))
        A = sp.coo_matrix((np.concatenate(vals_l), (np.concatenate(rows_l), np.concatenate(cols_l))),
                          shape=(nn + ns, nn + ns)).tocsr()
        A.sum_duplicates()
        return A

    def rhs(self, f):
        """b[ρ] .= f[ρ] ./ ε0 (:375) over the node block, then the σ block."""
        f = np.asarray(f, float).ravel(order="F")
        b = self.b.copy()
        b[self.rho_dof] = f[self.rho_dof] / self.eps0
        return np.concatenate([b, np.asarray(self.sig_b, float)])

    DENSE_MAX = 4096

    def factorize(self):
        """LU of the assembled system (the reference's ``A\\b``): dense LAPACK
        getrf/getrs up to DENSE_MAX unknowns, sparse LU beyond.  Rows are
        equilibrated first (identity Dirichlet rows sit next to 1/Δx² stencil
        rows) and solve() adds one step of FP64 iterative refinement, so the
        oracle returns the solution of the reference's system to full FP64
        accuracy.  Singular (no pinned row, zero row sums) -> bordered
        mean-zero system."""
        import scipy.sparse as sp
        import scipy.sparse.linalg as sla
        A = self.matrix()
        self.A = A
        n = A.shape[0]
        nn = self.nn
        ident = (self.C[:, 0] == 1.0) & np.all(self.C[:, 1:] == 0.0, axis=1)
        if self.sig_cols.shape[1]:
            ident &= np.all(self.sig_cols == 0.0, axis=1)
        rs = np.abs(np.asarray(A[:nn, :nn].sum(axis=1)).ravel())
        self.singular = (not ident.any()) and rs.max() <= 1e-12 * np.abs(self.C[:, 0]).max()
        if self.singular:
            one = np.zeros((n, 1))
            one[:nn] = 1.0
            A = sp.bmat([[A, sp.csr_matrix(one)], [sp.csr_matrix(one.T), None]]).tocsr()
        self.Afull = A
        self.rowscale = 1.0 / np.maximum(abs(A).max(axis=1).toarray().ravel(), 1e-300)
        As = sp.diags(self.rowscale) @ A
        if As.shape[0] <= self.DENSE_MAX:
            import scipy.linalg as la
            self.dense_lu = la.lu_factor(As.toarray())
            self.lu = None
        else:
            self.dense_lu = None
            self.lu = sla.splu(As.tocsc())

    def _lu_solve(self, b):
        bs = self.rowscale * b
        if self.dense_lu is not None:
            import scipy.linalg as la
            return la.lu_solve(self.dense_lu, bs)
        return self.lu.solve(bs)

    def solve(self, f):
        """calculate_electric_potential(ps, f) (:372-378): returns ϕ (nx,ny)."""
        if not hasattr(self, "A"):
            self.factorize()
        b = self.rhs(f)
        if self.singular:
            b = np.concatenate([b, [0.0]])
        x = self._lu_solve(b)
        x = x + self._lu_solve(b - self.Afull @ x)
        self.x = x[: self.nn + len(self.sig_b)]
        return self.x[: self.nn].reshape((self.nx, self.ny), order="F")

    def residual(self, phi, f):
        x = np.concatenate([np.asarray(phi).ravel(order="F"), np.asarray(self.sig_b, float)])
        b = self.rhs(f)
        r = b - self.A @ x
        return np.linalg.norm(r) / max(np.linalg.norm(b), 1e-300)


# ----------------------------------------------------------------------------
# The time loop body of ParticleInCell.solve (ParticleInCell.jl:102-135)
# ----------------------------------------------------------------------------

class SpeciesStore:
    """KineticSpecies{2,3} host store (pic/kinetic.jl:1-18): (cap,2)/(cap,3) F-order."""

    def __init__(self, q, m, w0, cap, x, v):
        self.q, self.m, self.w0, self.cap = q, m, w0, cap
        self.x = np.zeros((cap, 2), order="F")
        self.v = np.zeros((cap, 3), order="F")
        n = len(x)
        self.x[:n] = x
        self.v[:n] = v
        self.np = n
        self.bnd = (0, 0)       # after_push per axis: 0 none, 1 wrap!, 2 discard!
        self.absorbed = [0, 0, 0, 0]


class PicOracle:
    """MCC sets -> advance! every species -> circuit -> density/ρ -> ϕ -> E,
    each stage by the restatements above."""

    def __init__(self, nx, ny, dx, dy, eps0, bcs=(0, 0, 0, 0)):
        self.nx, self.ny, self.dx, self.dy, self.bcs = nx, ny, dx, dy, bcs
        self.ps = PoissonOracle(nx, ny, dx, dy, eps0)
        self.species = []
        self.mccs = []          # (MCCOracle, source index, product index or None, gas density)
        self.circuit = None
        self.E = np.zeros((nx, ny, 3), order="F")
        self.phi = np.zeros((nx, ny), order="F")
        self.rho = np.zeros((nx, ny), order="F")
        self.background = None
        self.counts = []

    def add_species(self, q, m, w0, cap, x, v, bnd=(0, 0)):
        s = SpeciesStore(q, m, w0, cap, x, v)
        s.bnd = bnd
        self.species.append(s)
        return len(self.species) - 1

    def add_mcc(self, mcc, src, prod, gas_n):
        self.mccs.append((mcc, src, prod, np.asfortranarray(gas_n, dtype=float)))
        self.counts.append(np.zeros(mcc.N, dtype=np.int64))

    def drive_dirichlet(self, nodes, amp, freq, phase=0.0, dc=0.0):
        """A problem's iteration hook calling apply_dirichlet(solver, nodes, V(t))
        after step n-1 (problem/11_rf_discharge.jl:93): the solve of step n
        (n >= 2) uses V((n-2)Δt)."""
        self.drives = getattr(self, "drives", []) + [(np.asarray(nodes, bool), amp, freq, phase, dc)]
        self.nstep = getattr(self, "nstep", 0)

    def set_circuit(self, R, L, C, amp, freq, dc, dof, pos_ref, neg_ref, area, scale=1.0, wall=0):
        """advance!(::CircuitRLC) (circuit_coupling.jl:35-43, Circuit.jl:117-136);
        pos_ref/neg_ref: (i, j) 0-based reference nodes; wall: discard! wall whose
        absorbed charge lands on the floating electrode (0 = x-low)."""
        self.circuit = dict(R=R, L=L, C=C, amp=amp, freq=freq, dc=dc, dof=dof, pos=pos_ref, neg=neg_ref,
                            area=area, scale=scale, wall=wall, state=np.zeros(3), absorbed_seen=None)

    def step(self, dt, seed):
        nx, ny, dx, dy = self.nx, self.ny, self.dx, self.dy
        for k, (m, si, pi, gas) in enumerate(self.mccs):
            S = self.species[si]
            P = self.species[pi] if pi is not None else None
            snp, pnp, c = m.perform(self.E, gas, dx, dy, dt, S.x, S.v, S.np, seed + 7919 * k,
                                    None if P is None else P.x, None if P is None else P.v,
                                    0 if P is None else P.np)
            S.np = snp
            if P is not None:
                P.np = pnp
            self.counts[k] += c
        for S in self.species:
            n = S.np
            x = np.asfortranarray(S.x[:n])
            v = np.asfortranarray(S.v[:n])
            pu = grid_to_particle(self.E, dx, dy, x)
            push_cartesian(x, v, pu, None, S.q / S.m, dt)
            for d, (mode, nn_, h) in enumerate(((S.bnd[0], nx, dx), (S.bnd[1], ny, dy))):
                if mode == 2:
                    wg = np.full(len(x), S.w0)
                    npn, lo, hi = discard(x, v, wg, None, S.w0, d, nn_, h)
                    x, v = np.asfortranarray(x[:npn]), np.asfortranarray(v[:npn])
                    S.absorbed[2 * d] += lo
                    S.absorbed[2 * d + 1] += hi
            for d, (mode, nn_, h) in enumerate(((S.bnd[0], nx, dx), (S.bnd[1], ny, dy))):
                if mode == 1:
                    wrap(x, d, nn_, h)
            S.np = len(x)
            S.x[:S.np] = x
            S.v[:S.np] = v
        if self.circuit is not None:
            c = self.circuit
            vext = self.phi[c["pos"]] - self.phi[c["neg"]]
            st = c["state"]
            vsrc = c["amp"] * np.sin(2 * np.pi * c["freq"] * st[2]) + c["dc"]
            c["state"] = advance_circuit(c["R"], c["L"], c["C"], st, vext, vsrc, dt)
            ds = -dt * c["state"][0] / c["area"] * c["scale"]
            seen = c["absorbed_seen"] or [0] * len(self.species)
            for s, S in enumerate(self.species):
                ds += S.q * S.w0 * (S.absorbed[c["wall"]] - seen[s]) / c["area"]
            c["absorbed_seen"] = [S.absorbed[c["wall"]] for S in self.species]
            self.ps.set_sigma(c["dof"], self.ps.sig_b[c["dof"] - 1] + ds)
            c["vext"] = vext
        rho = np.zeros((nx, ny), order="F")
        V = cell_volume(nx, ny, dx, dy, self.bcs)
        for S in self.species:
            u = particle_to_grid(nx, ny, dx, dy, S.x[:S.np], None, S.w0)
            rho += S.q * (u / V)
        if self.background is not None:
            rho += self.background
        self.rho = rho
        self.nstep = getattr(self, "nstep", 0) + 1
        if self.nstep >= 2:
            for mask, amp, freq, phase, dc in getattr(self, "drives", []):
                self.ps.apply_dirichlet(mask, amp * np.sin(2 * np.pi * freq * (self.nstep - 2) * dt + phase) + dc)
        self.phi = self.ps.solve(-rho)
        self.E = electric_field(self.phi, dx, dy)
