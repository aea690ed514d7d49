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


def slab(L, n_l, n_g, width=4.0, rows=4):
    """Periodic liquid slab in x (two flat interfaces at L/4 and 3L/4)."""
    x = np.arange(L, dtype=np.float64)
    prof = n_g + 0.5 * (n_l - n_g) * (np.tanh((x - L / 4) / width) - np.tanh((x - 3 * L / 4) / width))
    return np.tile(prof, (rows, 1))


def coexistence(G, stencil='D2E8', tau=1.0, L=128, width=4.0, guess=None, check_every=1000,
                max_steps=200000, tol=1e-12, device=0):
    """Bulk (rho_l, rho_g) of a flat interface at coupling G (FP64 plain path).

    Returns dict(rho_l, rho_g, steps, u_conv, finite)."""
    x, f = XIStencils['D2Q9'], FStencils[stencil]
    if guess is None:
        # a start in the two-phase region: the coexisting densities grow ~linearly with -G
        guess = (max(0.25, 4.6 + 1.4 * (-4.5 - G)), 0.2)
    n_l, n_g = guess
    dims = (L, 4)
    s = _lib.Sim(2, dims, x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], G, tau=tau, literals=_lib.LIT_EXACT,
                 device=device)
    s.set_density(slab(L, n_l, n_g, width))
    s.set_velocity(np.zeros(2 * s.V))
    s.init_populations()
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


def coexistence_many(Gs, stencil='D2E8', check_every=2000, max_steps=200000, tol=1e-11, L=128, device=0):
    """``coexistence`` for many couplings at once: every slab has its own
    handle and stream, so their (launch-bound) steps overlap on the GPU."""
    x, f = XIStencils['D2Q9'], FStencils[stencil]
    sims, out = [], []
    for G in Gs:
        s = _lib.Sim(2, (L, 4), x['XIs'], x['Ws'], x['c2'], f['Es'], f['Ws'], G, literals=_lib.LIT_EXACT,
                     device=device)
        s.set_density(slab(L, max(0.25, 4.6 + 1.4 * (-4.5 - G)), 0.2))
        s.set_velocity(np.zeros(2 * s.V))
        s.init_populations()
        s.compute_moments()
        s.check_u()
        sims.append(s)
        out.append(dict(G=float(G), steps=0, u_conv=float('nan'), status='running'))
    running = list(range(len(Gs)))
    while running:
        for i in running:
            sims[i].step(check_every, sync=False)
        for i in list(running):
            s = sims[i]
            s.compute_moments()
            uc, _ = s.check_u()
            out[i]['steps'] += check_every
            out[i]['u_conv'] = uc
            if not np.isfinite(uc) or not s.density_finite()[0]:
                out[i]['status'] = 'diverged'
            elif uc < tol:
                out[i]['status'] = 'converged'
            elif out[i]['steps'] >= max_steps:
                out[i]['status'] = 'max_steps'
            if out[i]['status'] != 'running':
                running.remove(i)
    for i, s in enumerate(sims):
        n = s.get_density().reshape(4, L)
        out[i]['rho_l'], out[i]['rho_g'] = float(n[0, L // 2]), float(n[0, 0])
        s.close()
    return out


def run_sweep(n=64, r_min=8, seed=2024, G_range=(-6.0, -4.5), stencil='D2E8', check_every=500, tol32=1e-5,
              tol64=1e-9, max_steps=100000, plain=True, device=0, init=None):
    """The ragged droplet sweep: radii r_min .. r_min+n-1, box 4R rounded up to
    32, G uniform in G_range (seeded), densities from the coexistence runs;
    batched FP32 run vs the plain FP64 path droplet by droplet."""
    rng = np.random.default_rng(seed)
    radii = list(range(r_min, r_min + n))
    Gs = rng.uniform(G_range[0], G_range[1], n)
    t0 = time.perf_counter()
    coex = coexistence_many(Gs, stencil=stencil, device=device)
    t_coex = time.perf_counter() - t0
    ok = [i for i, c in enumerate(coex) if c['status'] != 'diverged' and np.isfinite(c['rho_l'])]
    unstable = [dict(R=radii[i], G=float(Gs[i]), reason='flat interface diverged') for i in range(n) if i not in ok]
    rl = [coex[i]['rho_l'] for i in ok]
    rg = [coex[i]['rho_g'] for i in ok]
    sw = ragged_sweep([radii[i] for i in ok], [float(Gs[i]) for i in ok], rl, rg, stencil=stencil,
                      check_every=check_every, tol=tol32, max_steps=max_steps, device=device,
                      init=None if init is None else [init[i] for i in ok])
    res = dict(config=dict(n=n, radii=[r_min, r_min + n - 1], box='4R rounded up to 32', G_range=list(G_range),
                           seed=seed, stencil=stencil, tau=1.0, check_every=check_every, tol_fp32=tol32,
                           tol_fp64=tol64, criterion='u_conv = sum|u(t)-u(t-K)|/V (CheckUConvergenceSCMP)'),
               coexistence_wall_s=t_coex, unstable=unstable, batch=sw,
               coexistence=[coex[i] for i in ok])
    if plain:
        runs = []
        t1 = time.perf_counter()
        for j, i in enumerate(ok):
            runs.append(plain_run(radii[i], float(Gs[i]), rl[j], rg[j], stencil=stencil, check_every=check_every,
                                  tol=tol64, max_steps=max_steps, device=device))
        res['plain'] = runs
        res['plain_wall_s'] = time.perf_counter() - t1
    return res


# late import (batch imports MultiPhase, which imports this package's _lib)
from .batch import Batch as Batch_  # noqa: E402
