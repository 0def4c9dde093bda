"""FiniteDifferenceMethod mirror (FiniteDifferenceMethod/src/generalized_poisson.jl).

The solver lives on the device of its grid; the operator is assembled by the
same row operations as the reference and solved in FP64 to a relative
residual tolerance (see iskra_gb300/csrc/poisson.cu).
"""
from __future__ import annotations

import numpy as np

from . import _lib


class PoissonSolver:
    def __init__(self, grid, eps0):
        self.grid = grid
        self.ε0 = eps0
        self.ctx = grid.device
        self.ctx.poisson_create(eps0)
        self.rtol = 1e-8
        self.maxit = 10000
        self.iterations = 0
        self.relres = 0.0


def create_poisson_solver(grid, eps0):
    """create_poisson_solver(grid::CartesianGrid{2}, ε0) (:27-30)."""
    return PoissonSolver(grid, eps0)


def apply_dirichlet(ps, nodes, phi0):
    """apply_dirichlet(ps, nodes::BitArray, ϕ0) (:205-215)."""
    ps.ctx.apply_dirichlet(nodes, float(phi0))


def apply_periodic(ps, axis):
    """apply_periodic(ps::PoissonSolver{:xy,2}, axis) (:286-324)."""
    ps.ctx.apply_periodic(int(axis))


def add_new_dof(ps, symbol="σ"):
    """add_new_dof(ps, :σ) (:217-230); returns the 1-based dof index."""
    if symbol not in ("σ", "sigma"):
        raise ValueError("only the σ dof is supported")
    return ps.ctx.add_dof()


def apply_neumann(ps, nodes, dof):
    """apply_neumann(ps::PoissonSolver{:xy,2}, nodes, dof) (:235-269)."""
    ps.ctx.apply_neumann(nodes, int(dof))


def get_rhs(ps, symbol, dof):
    """get_rhs(ps, :σ, dof) (:367-370) -- value of the σ right-hand side."""
    return ps.ctx.get_sigma(dof)


def set_rhs(ps, symbol, dof, value):
    ps.ctx.set_sigma(dof, float(value))


def calculate_electric_potential(ps, f=None):
    """calculate_electric_potential(ps, f) (:372-378).  With f=None the device
    charge density is used (f = -ρ, as ParticleInCell.solve passes it)."""
    if f is None:
        ps.iterations, ps.relres = ps.ctx.solve(ps.rtol, ps.maxit)
        return ps.ctx.field(_lib.FIELD_PHI)
    phi, ps.iterations, ps.relres = ps.ctx.solve_host(np.asarray(f, float), ps.rtol, ps.maxit)
    return phi


def calculate_electric_field(ps, phi=None):
    """calculate_electric_field(ps, ϕ) (:382-410) of the last solve (FP64)."""
    return ps.ctx.field(_lib.FIELD_E)


def calculate_magnetic_field(ps):
    """calculate_magnetic_field (:412-419): identically zero."""
    nx, ny = ps.grid.n
    return np.zeros((nx, ny, 3), order="F")
