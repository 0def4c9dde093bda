"""Circuit mirror (Circuit/src/Circuit.jl) coupled to a floating electrode
(ParticleInCell/src/pic/circuit_coupling.jl).  The RLC state lives on the
device and advances in FP64 inside the step."""
from __future__ import annotations

import math


class CircuitRLC:
    def __init__(self, R, L, C, amp, freq, dc=0.0):
        self.R, self.L, self.C = R, L, C
        self.amp, self.freq, self.dc = amp, freq, dc
        self.ctx = None

    def V(self, t):
        return self.amp * math.sin(2 * math.pi * self.freq * t) + self.dc


def rlc(R, L, C, amp=0.0, freq=0.0, dc=0.0):
    """rlc(@netlist ...) (Circuit.jl:56-64) for a series R-L-C with a sine source."""
    return CircuitRLC(R, L, C, amp, freq, dc)


def damping_factor(R, L, C):
    """damping_factor (Circuit.jl:65)."""
    return (R / (2 * L)) * math.sqrt(L * C)


def resonant_frequency(L, C):
    """resonant_frequency (Circuit.jl:67)."""
    return 1 / math.sqrt(L * C) / (2 * math.pi)


def connect(cir, ps, sigma_dof, positive_nodes, negative_nodes, area, sigma_scale=1.0):
    """PlasmaDevice(positive floating electrode, negative fixed electrode)
    (circuit_coupling.jl:18-33) as the circuit's external device."""
    ps.ctx.circuit_create(cir.R, cir.L, cir.C, cir.amp, cir.freq, cir.dc, sigma_dof, positive_nodes,
                          negative_nodes, area, sigma_scale)
    cir.ctx = ps.ctx
    return cir


def advance(cir, phi, dt, config=None):
    """advance!(circuit::CircuitRLC, ϕ, Δt, config) (circuit_coupling.jl:35-43)."""
    cir.ctx.circuit_advance(dt)


def state(cir):
    return cir.ctx.circuit_state()
