"""iskra_gb300 -- GB300 (sm_103a) implementation of iskra's electrostatic PIC step.

Modules mirror the Julia reference's packages:
  regular_grids              RegularGrids
  particle_in_cell           ParticleInCell (species, advance!, density, solve)
  finite_difference_method   FiniteDifferenceMethod (Poisson solver, E field)
  chemistry                  Chemistry (CrossSection, MCC)
  circuit                    Circuit (RLC coupled to a floating electrode)
The compute runs in libiskra_gpu.so (include/iskra_gpu.h); device.Context is
the thin wrapper over that C ABI.
"""
from . import _lib
from ._lib import IskraError

__all__ = ["IskraError", "load_library"]


def load_library():
    """Loads (building if needed) libiskra_gpu.so and binds its C ABI."""
    return _lib.load()
