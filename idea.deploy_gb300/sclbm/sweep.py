"""Droplet sweeps: coexistence densities, batched FP32 droplets, FP64 plain runs.

* ``coexistence(G, ...)``: the plain method (FP64 GPU path) on a flat
  interface (a periodic slab, the reference's ``InitFlatInterface``,
  idpy/LBM/MultiPhase.py:1855-1895), stepped until the velocity stops
  changing; returns the bulk liquid and gas densities.
* ``ragged_sweep(...)``: droplets of radius R in boxes of side 4R rounded up
  to a multiple of 32, couplings G, densities from ``coexistence``; all run in
  one ``Batch`` (FP32-shifted storage, FP64 reductions) and are retired one by
  one as they converge.
* ``plain_runs(...)``: the same droplets one after another on the plain FP64
  GPU path, for the error and time-to-converge comparison.

Convergence is the reference's measure (CheckUConvergenceSCMP,
idpy/LBM/MultiPhaseLoopChecks.py:96-163): u_conv = sum_cells sum_d
|u(t) - u(t-K)| / V between two checks K steps apart, against a threshold.
A Shan-Chen droplet keeps steady spurious currents, so max|u| itself never
falls to zero; its value at convergence is reported.
"""
import math
import time

import numpy as np

from . import _lib
from .LBM import XIStencils, FStencils
from .profiles import droplet


def psi_exp(n):
    return np.exp(-1.0 / n)


def laplace_dp(n_in, n_out, G, c2=1.0 / 3, e2=1.0, psi=psi_exp):
    """p = c2 n + G e2 psi^2 / 2 (PBulk, idpy/LBM/MultiPhase.py:1759-1768)."""
    p = lambda n: c2 * n + 0.5 * G * e2 * psi(n) ** 2
    return p(n_in) - p(n_out), p(n_in), p(n_out)


def coexistence(G, stencil='D2E8', tau=1.0, L=128, width=None, guess=None, check_every=1000,
                max_steps=200000, tol=1e-13, device=0):
    """Bulk (rho_l, rho_g) of a flat interface at coupling G (FP64 plain path).

    Returns dict(rho_l, rho_g, steps, u_conv, finite)."""
    x, f = XIStencils['D2Q9'], FStencils[stencil]
    if guess is None:
        # a start in the two-phase region: the coexisting densities grow ~linearly with -G
        guess = (max(0.25, 4.6 + 1.35 * (-4.5 - G)), 0.2)
    n_l, n_g = guess
    dims = (L, 4)
    s = _lib.Sim(2, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], G, tau=tau, literals=_lib.LIT_EXACT,
                 device=device)
    s.init_flat(n_g, n_l, width or L / 2.0, 0, True)
    steps, uc, finite = 0, float('nan'), True
    s.compute_moments()
    s.check_u()
    while steps < max_steps:
        s.step(check_every)
        steps += check_every
        s.compute_moments()
        uc, _ = s.check_u()
        finite = s.density_finite()[0]
        if not finite or not np.isfinite(uc) or uc < tol:
            break
    n = s.get_density().reshape(4, L)
    s.close()
    return dict(rho_l=float(n[0, L // 2]), rho_g=float(n[0, 0]), steps=steps, u_conv=float(uc),
                finite=bool(finite and np.isfinite(n).all()))


def sweep_geometry(radii, multiple=32, factor=4):
    return [int(math.ceil(factor * R / multiple) * multiple) for R in radii]


def ragged_sweep(radii, G, rho_l, rho_g, stencil='D2E8', tau=1.0, width=2.0, check_every=500, tol=1e-7,
                 max_steps=200000, noise=0.0, seed=0, device=0, init=None):
    """Run all droplets in one FP32 batch until each converges; returns a dict
    of per-droplet arrays and the wall time.  ``init`` may give initial
    density fields (e.g. a learned warm start) instead of the tanh profile."""
    boxes = sweep_geometry(radii)
    sizes = [(L, L) for L in boxes]
    rho0 = [0.5 * (a + b) for a, b in zip(rho_l, rho_g)]
    t0 = time.perf_counter()
    b = Batch_(XIStencils['D2Q9'], FStencils[stencil], sizes, G, rho0, tau=tau, device=device)
    for i, (R, L) in enumerate(zip(radii, boxes)):
        n0 = init[i] if init is not None else droplet((L, L), R, rho_l[i], rho_g[i], width, seed + i, noise)
        b.set_density(i, n0)
    b.init_populations()
    n = len(radii)
    active = np.ones(n, np.int32)
    steps_done = np.zeros(n, np.int64)
    u_conv = np.full(n, np.nan)
    max_u = np.full(n, np.nan)
    status = np.array(['running'] * n, dtype=object)
    b.check()  # u_old := u of the initial state
    total = 0
    while active.any() and total < max_steps:
        b.step(check_every, sync=False)
        total += check_every
        uc, mu, m = b.check()
        for i in np.nonzero(active)[0]:
            u_conv[i], max_u[i] = uc[i], mu[i]
            if not (np.isfinite(uc[i]) and np.isfinite(m[i])):
                status[i], active[i] = 'diverged', 0
            elif uc[i] < tol:
                status[i], active[i] = 'converged', 0
        steps_done[:] = b.steps()
        if not active.all():
            b.set_active(active)
    wall = time.perf_counter() - t0
    dp, n_in, n_out = [], [], []
    for i, L in enumerate(boxes):
        nf = b.get_density(i)
        ni, no = nf[L // 2, L // 2], nf[L - 1, L - 1]
        n_in.append(ni)
        n_out.append(no)
        dp.append(laplace_dp(ni, no, G[i])[0])
    b.close()
    status[status == 'running'] = 'max_steps'
    return dict(radii=np.array(radii), boxes=np.array(boxes), G=np.array(G), steps=steps_done, u_conv=u_conv,
                max_u=max_u, status=status, dp=np.array(dp), n_in=np.array(n_in), n_out=np.array(n_out),
                wall_s=wall)


def plain_run(R, G, rho_l, rho_g, stencil='D2E8', tau=1.0, width=2.0, check_every=500, tol=1e-7,
              max_steps=200000, noise=0.0, seed=0, device=0):
    """One droplet on the plain FP64 GPU path (exact coefficients), same criterion."""
    L = sweep_geometry([R])[0]
    x, f = XIStencils['D2Q9'], FStencils[stencil]
    t0 = time.perf_counter()
    s = _lib.Sim(2, (L, L), x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], G, tau=tau, literals=_lib.LIT_EXACT,
                 device=device)
    s.set_density(droplet((L, L), R, rho_l, rho_g, width, seed, noise))
    s.set_velocity(np.zeros(2 * s.V))
    s.init_populations()
    s.compute_moments()
    s.check_u()
    steps, uc, status = 0, float('nan'), 'max_steps'
    while steps < max_steps:
        s.step(check_every)
        steps += check_every
        s.compute_moments()
        uc, mu = s.check_u()
        if not np.isfinite(uc) or not s.density_finite()[0]:
            status = 'diverged'
            break
        if uc < tol:
            status = 'converged'
            break
    nf = s.get_density().reshape(L, L)
    s.close()
    ni, no = nf[L // 2, L // 2], nf[L - 1, L - 1]
    return dict(R=R, L=L, steps=steps, u_conv=uc, status=status, dp=laplace_dp(ni, no, G)[0], n_in=ni, n_out=no,
                wall_s=time.perf_counter() - t0)


# late import (batch imports MultiPhase, which imports this package's _lib)
from .batch import Batch as Batch_  # noqa: E402
