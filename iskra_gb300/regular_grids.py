"""RegularGrids mirror (RegularGrids/src/RegularGrids.jl).

create_uniform_grid(xs, ys; left, right, bottom, top) -> UniformGrid holding
the node counts, spacing, origin and side conditions.  The grid also owns the
device context that every GPU object built on it shares.
"""
from __future__ import annotations

import numpy as np


class UniformGrid:
    """UniformGrid{:xy,2} (RegularGrids.jl:7-15)."""

    def __init__(self, n, dh, bcs, origin):
        self.n = tuple(int(v) for v in n)
        self.Δh = tuple(float(v) for v in dh)
        self.bcs = bcs
        self.origin = tuple(float(v) for v in origin)
        self._ctx = None

    @property
    def size(self):
        return self.n

    def periodic_flags(self):
        (l, r), (b, t) = self.bcs
        return tuple(int(s == "periodic") for s in (l, r, b, t))

    @property
    def device(self):
        """The device context of this grid (created on first use)."""
        if self._ctx is None:
            from .device import Context
            self._ctx = Context(self.n[0], self.n[1], self.Δh[0], self.Δh[1], self.periodic_flags())
        return self._ctx


def create_uniform_grid(xx, yy, left="open", right="open", bottom="open", top="open"):
    """create_uniform_grid (RegularGrids.jl:55-69): Δ from the first two nodes."""
    xx = np.asarray(xx, dtype=float)
    yy = np.asarray(yy, dtype=float)
    nx, ny = len(xx), len(yy)
    dx = xx[1] - xx[0] if nx > 1 else 1.0
    dy = yy[1] - yy[0] if ny > 1 else 1.0
    return UniformGrid((nx, ny), (dx, dy), ((left, right), (bottom, top)), (xx[0], yy[0]))


def cell_volume(g: UniformGrid):
    """cell_volume(::CartesianGrid{2}) (RegularGrids.jl:26-38), host side."""
    dx, dy = g.Δh
    nx, ny = g.n
    V = np.zeros((nx, ny), order="F") + dx * dy
    (left, right), (bottom, top) = g.bcs
    if left != "periodic":
        V[0, :] *= 0.5
    if right != "periodic":
        V[nx - 1, :] *= 0.5
    if bottom != "periodic":
        V[:, 0] *= 0.5
    if top != "periodic":
        V[:, ny - 1] *= 0.5
    return V
