"""CPU oracle of the surface tracker -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` imports this module, as the checker of the tracker walk inside
the GPU push (``iskra_gb300/csrc/particles.cu`` ``track_path``,
``iskra_gb300/csrc/tracker.cu``).  FP64 restatement of
ParticleInCell/src/pic/surfaces/{build,track,check,hit}.jl and the electrode
hit! methods of ParticleInCell/src/pic/circuit_coupling.jl, for 2D grids:

* surfaces are keyed by ordered pairs of 1-based cells, (ij, kl) -> surface,
  built by build_default_surface! (build.jl:31-44, get! on an empty dict) and
  build_surface_lookup! (build.jl:46-60, later calls replace earlier ones);
* track! (track.jl:39-52) records the particles whose cell (particle_cell,
  f = 1 + x / Δh) is either side of some key;
* check! (check.jl:18-68) walks each record from its old cell and offsets
  with the pushed velocity; hit! (hit.jl, circuit_coupling.jl:45-63)
  absorbs, reflects (position mirrored, normal velocity flipped, tracking
  continues from the near side of the edge, scattered!) or does nothing
  (periodic).

Parity is unpinned: the reference ships no tests or fixtures for the tracker
(ParticleInCell/test/runtests.jl holds a single ``@test true``), so this
restatement is checked against the reference source by reading and against
hand-computed trajectories in tests/test_tracker_oracle_cpu.py.  The one
generalisation: the reference walks both axes with Δh = Δx; here the y axis
uses Δy (identical for the square cells of every reference problem).
"""
from __future__ import annotations

import numpy as np

ABSORB, REFLECT, PERIODIC, FIXED, FLOATING = 1, 2, 3, 4, 5


class Tracker:
    """SurfaceTracker{2}: surfaces[(ij, kl)] = index into kinds."""

    def __init__(self, nx, ny, default_kind=ABSORB):
        self.nx, self.ny = nx, ny
        self.kinds = [default_kind]
        self.surfaces = {}
        # build_default_surface! (build.jl:36-44)
        for i in range(1, nx):
            self.surfaces.setdefault(((i, 1), (i, 0)), 0)
            self.surfaces.setdefault(((i, ny - 1), (i, ny)), 0)
        for j in range(1, ny):
            self.surfaces.setdefault(((1, j), (0, j)), 0)
            self.surfaces.setdefault(((nx - 1, j), (nx, j)), 0)
        self._cells = None

    def add(self, bcs, kind):
        """build_surface_lookup! (build.jl:46-60) with nodes bcs (nx, ny) bool
        (0-based array, 1-based cells)."""
        f = len(self.kinds)
        self.kinds.append(kind)
        b = np.asarray(bcs, bool)
        for i in range(1, self.nx):
            for j in range(1, self.ny):
                a_, b_ = b[i - 1, j - 1], b[i, j - 1]
                c_, d_ = b[i, j], b[i - 1, j]
                if a_ and b_:
                    self.surfaces[((i, j), (i, j - 1))] = f
                if b_ and c_:
                    self.surfaces[((i, j), (i + 1, j))] = f
                if c_ and d_:
                    self.surfaces[((i, j), (i, j + 1))] = f
                if d_ and a_:
                    self.surfaces[((i, j), (i - 1, j))] = f
        self._cells = None
        return f

    def tracked_cells(self):
        """The cells `(i, j) ∈ st` holds for (track.jl:19-26)."""
        if self._cells is None:
            s = set()
            for ij, kl in self.surfaces:
                s.add(ij)
                s.add(kl)
            self._cells = s
        return self._cells


def particle_cell(x, y, dx, dy):
    """particle_cell (ParticleInCell.jl:28-35) with Δh = (Δx, Δy): 1-based."""
    fx, fy = 1.0 + x / dx, 1.0 + y / dy
    i, j = int(np.floor(fx)), int(np.floor(fy))
    return i, j, fx - i, fy - j


def check_step(pt, vx, vy, dx, dy):
    """check(pt::TrackedParticle{2}, pv, Δh) (check.jl:18-37); pt = (Δt, (i, j),
    (hx, hy)).  Returns the next record (the same when the particle stays)."""
    t, (i, j), (hx, hy) = pt
    ddx = dx * (1 - hx) if vx > 0 else dx * hx
    ddy = dy * (1 - hy) if vy > 0 else dy * hy
    tx = ddx / abs(vx) if vx != 0 else np.inf
    ty = ddy / abs(vy) if vy != 0 else np.inf
    if t < tx and t < ty:
        return pt
    if tx < ty:
        return (t - tx, (i + 1, j), (0.0, hy + vy * tx / dy)) if vx > 0 else \
               (t - tx, (i - 1, j), (1.0, hy + vy * tx / dy))
    return (t - ty, (i, j + 1), (hx + vx * ty / dx, 0.0)) if vy > 0 else \
           (t - ty, (i, j - 1), (hx + vx * ty / dx, 1.0))


def advance_tracked(tr: Tracker, x0, v1, dt, dx, dy, qw=0.0, areas=None):
    """track! before and check! after one push, for particles at x0 (np, 2)
    before the push with pushed velocities v1 (np, >=2).  The pushed positions
    are x0 + v1 dt (the Boris push, pushers.jl:37-50).  Returns (x, v,
    absorbed mask, hits per surface, dσ per surface); dσ = q w hits / area for
    floating electrodes (circuit_coupling.jl:45-55).  Loops in Python: small
    cases only."""
    x0 = np.asarray(x0, float)
    v = np.array(v1, float, copy=True)
    x = x0 + v[:, :2] * dt
    absorbed = np.zeros(len(x0), bool)
    hits = np.zeros(len(tr.kinds), np.int64)
    cells = tr.tracked_cells()
    for p in range(len(x0)):
        i, j, hx, hy = particle_cell(x0[p, 0], x0[p, 1], dx, dy)
        if (i, j) not in cells:
            continue
        pt = (dt, (i, j), (hx, hy))
        for _ in range(64):
            pt2 = check_step(pt, v[p, 0], v[p, 1], dx, dy)
            ij, ij2 = pt[1], pt2[1]
            if ij == ij2:
                break
            f = tr.surfaces.get((ij, ij2))
            if f is None:
                pt = pt2
                continue
            kind = tr.kinds[f]
            if kind == PERIODIC:
                break
            if kind != REFLECT:
                absorbed[p] = True
                hits[f] += 1
                break
            # ReflectiveSurface hit! (hit.jl:40-56) then scattered! (:17-25)
            t2, (i2, j2), (hx2, hy2) = pt2
            n = (i2 - ij[0], j2 - ij[1])
            x[p] -= v[p, :2] * t2
            if n[0] != 0:
                v[p, 0] = -v[p, 0]
            if n[1] != 0:
                v[p, 1] = -v[p, 1]
            x[p] += v[p, :2] * t2
            ii, jj, hxx, hyy = i2, j2, hx2, hy2
            if hx2 == 0.0:
                ii, hxx = i2 - 1, 1.0
            if hx2 == 1.0:
                ii, hxx = i2 + 1, 0.0
            if hy2 == 0.0:
                jj, hyy = j2 - 1, 1.0
            if hy2 == 1.0:
                jj, hyy = j2 + 1, 0.0
            pt = (t2, (ii, jj), (hxx, hyy))
    dsig = np.zeros(len(tr.kinds))
    if areas is not None:
        for f, a in areas.items():
            dsig[f] = qw * hits[f] / a
    return x, v, absorbed, hits, dsig


def decision_margin(tr: Tracker, x0, v1, dt, dx, dy):
    """Smallest relative gap of the walk's comparisons (remaining time against
    the edge times, the two edge times, the crossing point against the cell
    corners) per particle; tests keep only well-separated particles, whose
    outcome FP32 arithmetic reproduces."""
    x0 = np.asarray(x0, float)
    out = np.full(len(x0), np.inf)
    cells = tr.tracked_cells()
    v1 = np.asarray(v1, float)
    for p in range(len(x0)):
        i, j, hx, hy = particle_cell(x0[p, 0], x0[p, 1], dx, dy)
        if (i, j) not in cells:
            continue
        vx, vy = v1[p, 0], v1[p, 1]
        t = dt
        m = np.inf
        for _ in range(4):
            ddx = dx * (1 - hx) if vx > 0 else dx * hx
            ddy = dy * (1 - hy) if vy > 0 else dy * hy
            tx = ddx / abs(vx) if vx != 0 else np.inf
            ty = ddy / abs(vy) if vy != 0 else np.inf
            for a, b in ((t, tx), (t, ty), (tx, ty)):
                if np.isfinite(a) and np.isfinite(b):
                    m = min(m, abs(a - b) / dt)
            m = min(m, hx, 1 - hx, hy, 1 - hy) if (hx not in (0.0, 1.0) and hy not in (0.0, 1.0)) else m
            if t < tx and t < ty:
                break
            if tx < ty:
                t -= tx
                hy += vy * tx / dy
                hx = 0.0 if vx > 0 else 1.0
                m = min(m, hy, 1 - hy)
            else:
                t -= ty
                hx += vx * ty / dx
                hy = 0.0 if vy > 0 else 1.0
                m = min(m, hx, 1 - hx)
        out[p] = m
    return out
