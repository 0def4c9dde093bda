"""Micro-benchmarks of the learned warm start and the multigrid-CG step (one GPU).

  python -m iskra_gb300.lws_bench net [--size 1024] [--reps 20]
      forward pass and loss + gradient of the network on a size x size image
      (host-timed, including the image copies)
  python -m iskra_gb300.lws_bench step [--size 1024] [--particles 4194304] [--steps 2]
      steps of the 2D argon discharge at size x size nodes with the
      multigrid-preconditioned CG solve and the network's warm start in use
      mode; the measured steps are bracketed by cudaProfilerStart/Stop (for
      `ncu --profile-from-start off`)

Both print one line of timings.  The profiles under profiles/ name the
command lines they ran.
"""
from __future__ import annotations

import argparse
import time

import numpy as np

QE, ME, KB, EPS0 = 1.602176634e-19, 9.1093837015e-31, 1.380649e-23, 8.8541878128e-12
M_AR = 39.948 * 1.66053906660e-27
DT, FREQ = 7.4e-11, 13.56e6


def net(size, reps):
    from .device import Context
    ctx = Context(size, size, 1e-4, 1e-4, (0, 0, 0, 0))
    ctx.lws_create(0, seed=3)
    rng = np.random.default_rng(11)
    x = rng.standard_normal((size, size)).astype(np.float32)
    t = (0.1 * rng.standard_normal((size, size))).astype(np.float32)
    for _ in range(3):
        ctx.lws_forward(x)
        ctx.lws_loss_grad(x, t)
    ctx.sync()
    t0 = time.perf_counter()
    for _ in range(reps):
        ctx.lws_forward(x)
    ctx.sync()
    t1 = time.perf_counter()
    for _ in range(reps):
        ctx.lws_loss_grad(x, t)
    ctx.sync()
    t2 = time.perf_counter()
    ctx.close()
    print(f"network {size}x{size}: forward {1e3 * (t1 - t0) / reps:.3f} ms, loss + gradient "
          f"{1e3 * (t2 - t1) / reps:.3f} ms per call (host timed, image copies included)")


def step(size, npart, steps):
    import torch
    from . import _lib
    from .device import Context
    dx = 1e-4
    L = (size - 1) * dx
    ctx = Context(size, size, dx, dx, (0, 0, 0, 0))
    sids = []
    for q, m, T in ((-QE, ME, 4.0), (QE, M_AR, 0.03)):
        sid = ctx.species_create(q, m, 1e15 * L * L / npart, int(npart * 1.25))
        ctx.set_boundary(sid, _lib.BND_DISCARD, _lib.BND_WRAP)
        src = ctx.source_create(sid, npart / DT, (L, L), np.sqrt(2 * T * QE / m))
        ctx.source_sample(src, DT, seed=11 + len(sids))
        sids.append(sid)
    ctx.poisson_create(EPS0)
    ctx.apply_periodic(1)
    left = np.zeros((size, size), bool)
    left[0, :] = True
    right = np.zeros((size, size), bool)
    right[-1, :] = True
    ctx.apply_dirichlet(left, 0.0)
    ctx.apply_dirichlet(right, 0.0)
    ctx.drive_dirichlet(left, 300.0, FREQ)
    method = ctx.set_method(2)
    ctx.lws_create(16, seed=5)
    ctx.lws_set_mode(harvest=True)
    for _ in range(12):
        ctx.step(DT, 1, seed=1, rtol=1e-8)
    ctx.lws_set_mode()
    ctx.lws_train(20, lr=1e-3, seed=1)
    ctx.lws_set_mode(use=True, smooth=0)
    for _ in range(3):
        ctx.step(DT, 1, seed=1, rtol=1e-8)
    ctx.sync()
    torch.cuda.profiler.start()
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.step(DT, 1, seed=1, rtol=1e-8)
    ctx.sync()
    t1 = time.perf_counter()
    torch.cuda.profiler.stop()
    it, rr = ctx.solve_info()
    ctx.close()
    print(f"step {size}x{size}, {npart} + {npart} particles, solver method {method}: "
          f"{1e3 * (t1 - t0) / steps:.3f} ms per step (host timed), last solve {it} iterations to relres {rr:.2e}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["net", "step"])
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--particles", type=int, default=1 << 22)
    ap.add_argument("--steps", type=int, default=2)
    a = ap.parse_args()
    if a.what == "net":
        net(a.size, a.reps)
    else:
        step(a.size, a.particles, a.steps)


if __name__ == "__main__":
    main()
