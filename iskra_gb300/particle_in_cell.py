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


# ---- sources (pic/sources.jl, problem/configuration.jl:89-93) ----------------
KB = 1.380649e-23


class MaxwellianSource:
    """MaxwellianSource{2,3}(rate, wx, wv; dx, dv) (sources.jl:8-22).  The
    device object is created when the source is first sampled for a species."""

    def __init__(self, rate, wx, wv, dx=None, dv=None):
        self.rate = float(rate)
        self.wx = np.asarray(wx, float).ravel()
        self.wv = np.asarray(wv, float).ravel()
        self.dx = np.zeros(2) if dx is None else np.asarray(dx, float).ravel()
        self.dv = np.zeros(3) if dv is None else np.asarray(dv, float).ravel()
        self.species = None
        self.index = None

    def _bind(self, species):
        if self.index is None:
            self.species = species
            self.index = species.ctx.source_create(species.sid, self.rate, self.wx, self.wv, self.dx, self.dv)
        elif species is not self.species:
            raise ValueError("a source feeds one species")
        return self.index


def thermal_speed(T, m):
    """thermal_speed (problem/configuration.jl:80-82): sqrt(2 kB T / m)."""
    return np.sqrt(2 * KB * T / m)


def create_thermalized_beam(species, x, vb, dx=None, T=300.0, rate=1.0):
    """create_thermalized_beam (problem/configuration.jl:89-93)."""
    vth = thermal_speed(T, species.m) * np.ones(3)
    src = MaxwellianSource(rate, x, vth, dx=dx, dv=vb)
    src.species = species
    return src


def sample(src: MaxwellianSource, species, dt, seed=0):
    """sample!(src, species, Δt) (sources.jl:24-34) on the device."""
    k = src._bind(species)
    species.ctx.source_sample(k, dt, seed)


def init(src: MaxwellianSource, species, dt, seed=0):
    """init(src, species, Δt) (ParticleInCell.jl:47-49)."""
    sample(src, species, dt, seed)


# ---- surfaces (pic/surfaces/build.jl:8-25, circuit_coupling.jl:4-16) --------
class Surface:
    kind = _lib.SURF_PERIODIC


class PeriodicSurface(Surface):
    """PeriodicSurface: hit! does nothing (hit.jl:26-31); tracking ends."""
    kind = _lib.SURF_PERIODIC


class AbsorbingSurface(Surface):
    """AbsorbingSurface: hit! removes the particle (hit.jl:33-39)."""
    kind = _lib.SURF_ABSORB


class ReflectiveSurface(Surface):
    """ReflectiveSurface: hit! mirrors the rest of the step (hit.jl:40-56)."""
    kind = _lib.SURF_REFLECT


@dataclass(eq=False)  # surfaces compare by identity, as the tracker's keys do
class FixedPotentialElectrode(Surface):
    """FixedPotentialElectrode (circuit_coupling.jl:4-8): absorbs (:57-63)."""
    phi: float = 0.0
    area: float = 0.0
    kind = _lib.SURF_FIXED


@dataclass(eq=False)
class FloatingPotentialElectrode(Surface):
    """FloatingPotentialElectrode (circuit_coupling.jl:10-15): absorbs and adds
    q w / area to its σ dof (:45-55)."""
    dof: int = 0
    area: float = 0.0
    kind = _lib.SURF_FLOATING


def create_periodic_surface():
    return PeriodicSurface()


def create_absorbing_surface():
    return AbsorbingSurface()


def create_reflective_surface():
    return ReflectiveSurface()


class SurfaceTracker:
    """SurfaceTracker{2} (build.jl:13-18) on the device of its grid: every push
    (advance, solve) walks the particles of cells next to a surface through
    check! and hit!."""

    def __init__(self, grid, ds):
        self.ctx = grid.device
        self.grid = grid
        self.ctx.tracker_create(ds.kind)
        self.surfaces = [ds]  # index = device surface index

    def index(self, ss):
        for k, x in enumerate(self.surfaces):
            if x is ss:
                return k
        raise KeyError("surface not tracked")

    def hits(self, ss, part):
        """Particles of `part` absorbed by surface `ss` so far."""
        return self.ctx.tracker_hits(self.index(ss), part.sid)


def create_surface_tracker(grid, ds=None):
    """create_surface_tracker(grid::CartesianGrid{2}, ds=AbsorbingSurface())
    (build.jl:91-97): the domain walls get surface ds."""
    return SurfaceTracker(grid, ds if ds is not None else AbsorbingSurface())


def track_surface(tracker: SurfaceTracker, bcs, ss: Surface):
    """track_surface!(tracker, bcs, ss) (build.jl:104-106): cell edges with both
    end nodes in bcs (bool (nx, ny)) become surface ss."""
    dof = getattr(ss, "dof", 0) if ss.kind == _lib.SURF_FLOATING else 0
    area = getattr(ss, "area", 0.0) if ss.kind == _lib.SURF_FLOATING else 0.0
    f = tracker.ctx.tracker_add_surface(np.asarray(bcs, bool), ss.kind, dof, area)
    tracker.surfaces.append(ss)
    assert f == len(tracker.surfaces) - 1
    return ss


def electrode_area(nodes, grid):
    """calculate_area (problem/configuration.jl:43-51): Δx Δz per node with a
    node to its +x, Δy Δz per node with a node to its +y (Δz = 1)."""
    m = np.asarray(nodes, bool)
    dx, dy = grid.Δh
    return float(dx * np.count_nonzero(m[:-1, :] & m[1:, :]) + dy * np.count_nonzero(m[:, :-1] & m[:, 1:]))


def create_electrode(nodes, config, fixed=False, sigma=0.0, phi=0.0):
    """create_electrode(nodes, config; fixed, σ, ϕ) (problem/configuration.jl:
    22-72): a fixed electrode is a Dirichlet node set at ϕ; a floating one a
    new σ dof with Neumann rows (σ = sigma).  Creates the tracker (absorbing
    walls) if the config has none and tracks the electrode surface."""
    from . import finite_difference_method as fdm
    if config.grid is None or config.solver is None:
        raise ValueError("create_electrode needs config.grid and config.solver")
    if config.tracker is None:
        config.tracker = create_surface_tracker(config.grid)
    nodes = np.asarray(nodes, bool)
    area = electrode_area(nodes, config.grid)
    if fixed:
        fdm.apply_dirichlet(config.solver, nodes, phi)
        el = FixedPotentialElectrode(phi=float(phi), area=area)
    else:
        dof = fdm.add_new_dof(config.solver, "σ")
        fdm.apply_neumann(config.solver, nodes, dof)
        fdm.set_rhs(config.solver, "σ", dof, sigma)
        el = FloatingPotentialElectrode(dof=dof, area=area)
    track_surface(config.tracker, nodes, el)
    return el


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
    for src in config.sources:  # sampled at the start of every step (:104-106)
        if src.species is None:
            raise ValueError("a source in config.sources needs its species (create_thermalized_beam)")
        ctx.source_every_step(src._bind(src.species), True)
    ctx.step(dt, int(timesteps), seed, rtol)
    ctx.sync()
