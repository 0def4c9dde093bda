"""CPU oracle of DSMC -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` imports this module, as the checker of the device DSMC
(``iskra_gb300/csrc/dsmc.cu``).  FP64 restatement of PIC.perform!(::Direct-
SimulationMonteCarlo, E, Δt, config) (Chemistry/src/dsmc.jl:86-138) for one
DSMC.ElasticCollision with perform! (:31-84, the vss_inv = 1 branch).
Declared deviations, shared with the device: the pair redraw of :112-114
applies when source and target are one species (the reference compares
indices of two different species); the unequal-weight branch updates the
target particle t (the reference writes target.v[s,:], :81).  Julia's random
stream cannot be reproduced: the number of pairs tried per cell and the
carried remainder are deterministic and compared exactly, the accepted
collisions statistically (parity unpinned otherwise).
"""
from __future__ import annotations

import numpy as np


def sgmax(g, sigma):
    """maximum(rate) * argmax(rate) (dsmc.jl:101, cross_section.jl:15-16)."""
    g, sigma = np.asarray(g, float), np.asarray(sigma, float)
    k = int(np.argmax(sigma))
    return sigma[k] * g[k]


def cells_of(x, dx, dy, nx):
    """0-based cell numbers i0 + nx j0 (particle_cell, ParticleInCell.jl:28-35)."""
    return np.floor(x[:, 0] / dx).astype(np.int64) + nx * np.floor(x[:, 1] / dy).astype(np.int64)


def pairs_and_remaining(Na, Nb, Wa, Wb, dx, dy, dt, sgm, same, remaining):
    """Per cell: floor(Nc) and the new remainder (dsmc.jl:94-117); cells with
    Na < 2 or Nb < 2 keep their remainder and try nothing."""
    Na, Nb = np.asarray(Na, float), np.asarray(Nb, float)
    Pab, Pba = (Wb / Wa, 1.0) if Wa > Wb else (1.0, Wa / Wb)
    na = Na * Wa / (dx * dy)
    Nc = na * Nb * dt * sgm
    Nc = Nc / (Pab + (Wb / Wa) * Pba)
    if not same:
        Nc = Nc * 2
    Nc = Nc + remaining
    act = (Na >= 2) & (Nb >= 2)
    fl = np.floor(Nc)
    new_rem = np.where(act, Nc - fl, remaining)
    return np.where(act, fl, 0).astype(np.int64), new_rem


def perform(xa, va, xb, vb, ma, mb, Wa, Wb, g, sigma, grid, dt, remaining, same=False, rng=None):
    """One perform! (Python loops; small cases).  Returns (va, vb, remaining,
    ν per cell)."""
    rng = np.random.default_rng(0) if rng is None else rng
    nx, ny, dx, dy = grid
    va, vb = np.array(va, float), (np.array(vb, float) if not same else None)
    if same:
        vb = va
    ca, cb = cells_of(xa, dx, dy, nx), cells_of(xb, dx, dy, nx)
    nn = nx * ny
    lists_a = [np.flatnonzero(ca == k) for k in range(nn)]
    lists_b = lists_a if same else [np.flatnonzero(cb == k) for k in range(nn)]
    Na = np.array([len(l) for l in lists_a])
    Nb = np.array([len(l) for l in lists_b])
    sgm = sgmax(g, sigma)
    npairs, rem = pairs_and_remaining(Na, Nb, Wa, Wb, dx, dy, dt, sgm, same, remaining)
    mr1, mr2 = ma / (ma + mb), mb / (ma + mb)
    nu = np.zeros(nn, np.int64)
    for k in range(nn):
        la, lb = lists_a[k], lists_b[k]
        for _ in range(npairs[k]):
            s = la[rng.integers(len(la))]
            t = lb[rng.integers(len(lb))]
            while same and t == s:
                t = lb[rng.integers(len(lb))]
            gv = va[s] - vb[t]
            gn = np.linalg.norm(gv)
            P = np.interp(gn, g, sigma) * gn / sgm
            if P < rng.random():
                continue
            vc = mr1 * va[s] + mr2 * vb[t]
            B = 2 * rng.random() - 1
            A = np.sqrt(1 - B * B)
            C = 2 * np.pi * rng.random()
            vr = gn * np.array([B, A * np.cos(C), A * np.sin(C)])
            if Wa == Wb:
                va[s] = vc + mr2 * vr
                vb[t] = vc - mr1 * vr
            else:
                R = rng.random()
                if Wb / Wa > R:
                    va[s] = vc + mr2 * vr
                if Wa / Wb > R:
                    vb[t] = vc - mr2 * vr
            nu[k] += 1
    return va, vb, rem, nu.reshape((nx, ny), order="F")
