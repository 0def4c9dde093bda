"""Host-side mirror logic of the tracker, electrodes and sources (no device):
calculate_area (problem/configuration.jl:43-51), thermal_speed
(configuration.jl:80-82), create_thermalized_beam (:89-93) and the surface
kinds of the tracker API."""
import types

import numpy as np

from iskra_gb300 import _lib
from iskra_gb300 import particle_in_cell as pic
from iskra_gb300.regular_grids import create_uniform_grid


def _calculate_area_literal(nodes, dx, dy):
    """calculate_area as the reference writes it (1-based loop over findall)."""
    nx, ny = nodes.shape
    area = 0.0
    for i, j in zip(*np.nonzero(nodes)):
        area += dx if (i + 1 < nx and nodes[i + 1, j]) else 0.0
        area += dy if (j + 1 < ny and nodes[i, j + 1]) else 0.0
    return area


def test_electrode_area_matches_the_reference_loop():
    g = create_uniform_grid(np.arange(12) * 0.1, np.arange(9) * 0.05)
    r = np.random.default_rng(0)
    for _ in range(5):
        m = r.random((12, 9)) < 0.4
        assert np.isclose(pic.electrode_area(m, g), _calculate_area_literal(m, 0.1, 0.05), rtol=0, atol=1e-12)
    m = np.zeros((12, 9), bool)
    m[0, 1:8] = True  # a wall segment of 7 nodes: 6 edges of Δy
    assert np.isclose(pic.electrode_area(m, g), 6 * 0.05)


def test_thermal_speed_and_beam():
    me = 9.1093837015e-31
    assert np.isclose(pic.thermal_speed(300.0, me), np.sqrt(2 * 1.380649e-23 * 300.0 / me))
    e = types.SimpleNamespace(m=me)
    src = pic.create_thermalized_beam(e, [0.1, 0.2], [1e3, 0.0, -1e3], T=2.0, rate=5e9)
    assert src.species is e and src.rate == 5e9
    assert np.allclose(src.wx, [0.1, 0.2]) and np.allclose(src.dx, [0.0, 0.0])
    assert np.allclose(src.wv, pic.thermal_speed(2.0, me)) and np.allclose(src.dv, [1e3, 0.0, -1e3])


def test_surface_kinds():
    assert pic.create_absorbing_surface().kind == _lib.SURF_ABSORB
    assert pic.create_reflective_surface().kind == _lib.SURF_REFLECT
    assert pic.create_periodic_surface().kind == _lib.SURF_PERIODIC
    assert pic.FixedPotentialElectrode().kind == _lib.SURF_FIXED
    assert pic.FloatingPotentialElectrode(dof=1, area=0.5).kind == _lib.SURF_FLOATING
