"""ParticleInCell mirror (ParticleInCell/src/ParticleInCell.jl and pic/*.jl).

KineticSpecies live in device memory (cell index + FP32 offsets + FP32
velocities, int64 fixed-point density).  advance / density / solve keep the
reference's names, argument meaning and step order; fields never leave the
device unless requested.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib


class KineticSpecies:
    """KineticSpecies{2,3} (pic/kinetic.jl:1-18) backed by the device store."""

    def __init__(self, name, N, q, m, w0, grid):
        self.name, self.q, self.m, self.w0 = name, float(q), float(m), float(w0)
        self.grid = grid
        self.ctx = grid.device
        self.capacity = int(N)
        self.sid = self.ctx.species_create(self.q, self.m, self.w0, self.capacity)

    @property
    def np(self):
        return self.ctx.count(self.sid)

    def load(self, x, v, wg=None, ids=None):
        """Sets the particles (x (np,2), v (np,3), Julia layout)."""
        self.ctx.upload(self.sid, x, v, wg, ids)

    def state(self):
        """(x, v, id) of the live particles, compacted."""
        return self.ctx.download(self.sid)


class FluidSpecies:
    """FluidSpecies (pic/fluid.jl:1-11): fixed node density n (nx, ny)."""

    def __init__(self, name, mu, q, m, n, T):
        self.name, self.μ, self.q, self.m, self.T = name, mu, float(q), float(m), float(T)
        self.n = np.asfortranarray(np.asarray(n, float))


def create_kinetic_species(name, N, q, m, weight, grid):
    """create_kinetic_species (problem/configuration.jl:141-148)."""
    return KineticSpecies(name, N, q, m, weight, grid)


def wrap(part, grid, dims=(1, 2)):
    """Registers wrap! (pic/surfaces/wrap.jl:20-33) as part of after_push."""
    _after_push(part, dims, _lib.BND_WRAP)


def discard(part, grid, dims=(1, 2)):
    """Registers discard! (pic/surfaces/wrap.jl:1-18) as part of after_push."""
    _after_push(part, dims, _lib.BND_DISCARD)


def _after_push(part, dims, mode):
    modes = list(getattr(part, "_bnd", [_lib.BND_NONE, _lib.BND_NONE]))
    for d in ((dims,) if isinstance(dims, int) else dims):
        modes[d - 1] = mode
    part._bnd = modes
    part.ctx.set_boundary(part.sid, modes[0], modes[1])


def advance(part: KineticSpecies, E=None, B=None, dt=1e-5, config=None):
    """advance!(::KineticSpecies, E, B, Δt, config) (ParticleInCell.jl:51-72):
    gather + Boris push + after_push on the device.  E (host (nx,ny,3)) is
    uploaded when given; otherwise the device field of the last solve is used.
    B must be zero (the reference's calculate_magnetic_field)."""
    if B is not None and np.any(np.asarray(B) != 0):
        raise ValueError("only B = 0 is supported (generalized_poisson.jl:412-419)")
    if E is not None:
        part.ctx.upload_E(E)
    part.ctx.advance(part.sid, dt)


def density(part, grid=None):
    """density(species, grid) (kinetic.jl:53 / fluid.jl:11)."""
    if isinstance(part, FluidSpecies):
        return part.n
    return part.ctx.density(part.sid)


@dataclass
class Config:
    """Config (problem/configuration.jl:5-15)."""
    solver: object = None
    pusher: object = None
    tracker: object = None
    interactions: list = field(default_factory=list)
    species: list = field(default_factory=list)
    sources: list = field(default_factory=list)
    circuit: object = None
    grid: object = None
    cells: object = None


def solve(config: Config, dt=1e-5, timesteps=200, seed=0, rtol=1e-8, background=None):
    """ParticleInCell.solve (ParticleInCell.jl:84-139): the time loop, run as
    device steps (MCC sets -> advance every kinetic species -> circuit ->
    density/ρ -> Poisson -> E), replayed as CUDA graphs.  `background` is a
    fixed charge density (a neutralising fluid species with constant n)."""
    ctx = config.grid.device
    if background is not None:
        ctx.set_background(background)
    ctx.step(dt, int(timesteps), seed, rtol)
    ctx.sync()
