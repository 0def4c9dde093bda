"""Chemistry mirror: cross sections and Monte Carlo collisions
(Chemistry/src/cross_section.jl, Chemistry/src/mcc.jl)."""
from __future__ import annotations

import numpy as np

from . import _lib


class CrossSection:
    """CrossSection(xs, ys): linear interpolation, flat extrapolation
    (cross_section.jl:3-14).  The device evaluates it; nodes are kept here."""

    def __init__(self, xs, ys):
        self.nodes = np.column_stack([np.asarray(xs, float), np.asarray(ys, float)])

    def __call__(self, e):
        return float(np.interp(e, self.nodes[:, 0], self.nodes[:, 1]))


class ElasticIsotropic:
    code = _lib.MCC_ELASTIC_ISOTROPIC
    energy = 0.0


class ElasticBackward:
    code = _lib.MCC_ELASTIC_BACKWARD
    energy = 0.0


class InelasticBackward:
    code = _lib.MCC_INELASTIC_BACKWARD
    energy = 0.0


class Excitation:
    code = _lib.MCC_EXCITATION

    def __init__(self, energy):
        self.energy = float(energy)


class Ionization:
    code = _lib.MCC_IONIZATION

    def __init__(self, energy):
        self.energy = float(energy)


class Reaction:
    """One line of @reactions (reactions.jl): rate, source + target --> products, type."""

    def __init__(self, rate: CrossSection, source, target, products=(), type=None):
        self.rate, self.source, self.target = rate, source, target
        self.products = list(products)
        self.type = type if type is not None else ElasticIsotropic()


class MonteCarloCollisions:
    def __init__(self, reactions):
        if not reactions:
            raise ValueError("empty reaction list")
        src = reactions[0].source
        tgt = reactions[0].target
        for r in reactions:
            if r.source is not src or r.target is not tgt:
                raise ValueError("one MCC set has one kinetic source and one fluid target (mcc.jl:36-39)")
        self.reactions = reactions
        self.source, self.target = src, tgt
        prods = [p for r in reactions for p in r.products if p is not src]
        self.product = prods[0] if prods else None
        ctx = src.ctx
        procs = [(r.type.code, r.type.energy, r.rate.nodes[:, 0], r.rate.nodes[:, 1]) for r in reactions]
        self.mid, self.max_σₜg = ctx.mcc_create(src.sid, procs, tgt.m, tgt.T, tgt.n, gas_q=tgt.q,
                                                product=self.product.sid if self.product is not None else -1)
        self.ctx = ctx
        self.N = len(reactions)
        self.step = 0


def mcc(reactions):
    """mcc(@reactions ...) (mcc.jl:313-320)."""
    return MonteCarloCollisions(list(reactions))


def perform(m: MonteCarloCollisions, E, dt, config=None, seed=0):
    """PIC.perform!(::MonteCarloCollisions, E, Δt, config) (mcc.jl:231-289) on
    the device E field.  Returns nothing; counts via collision_counts."""
    m.step += 1
    m.ctx.mcc_perform(m.mid, dt, seed, m.step)


def collision_counts(m: MonteCarloCollisions):
    return m.ctx.mcc_counts(m.mid, m.N)


class DirectSimulationMonteCarlo:
    """DirectSimulationMonteCarlo (dsmc.jl:15-22) of elastic collisions
    (DSMC.ElasticCollision, dsmc.jl:1-13) between kinetic species; one device
    set per collision."""

    def __init__(self, collisions):
        self.collisions = collisions
        self.sets = []
        for r in collisions:
            if r.products and any(p is not r.source and p is not r.target for p in r.products):
                raise ValueError("DSMC: only elastic collisions (the reference implements no other perform!)")
            ctx = r.source.ctx
            self.sets.append(ctx.dsmc_create(r.source.sid, r.target.sid, r.rate.nodes[:, 0], r.rate.nodes[:, 1]))
        self.ctx = collisions[0].source.ctx
        self.step = 0

    def nu(self):
        """The "nuDSMC" field of the last perform (sum over the collisions)."""
        return sum(self.ctx.dsmc_state(k)[1].astype(np.int64) for k in self.sets)


def dsmc(reactions):
    """dsmc(@reactions ...) (dsmc.jl:140-166): a Reaction per collision with
    kinetic source and target species."""
    return DirectSimulationMonteCarlo(list(reactions))


def perform_dsmc(d: DirectSimulationMonteCarlo, E, dt, config=None, seed=0):
    """PIC.perform!(::DirectSimulationMonteCarlo, E, Δt, config) (dsmc.jl:86-138)."""
    d.step += 1
    for k in d.sets:
        d.ctx.dsmc_perform(k, dt, seed, d.step)
